/*
 * sf_capi.h - C ABI of the GB300 (sm_103a) spatial-filtering hot path.
 *
 * One integration of int8 complex voltages, in the reference's packet layout,
 * goes through: correlation into int32 visibilities -> per-channel Hermitian
 * covariance -> eigendecomposition -> RFI-subspace projection (I - U U^H) ->
 * beamforming with projected weights (gains and fine-delay phasors folded in).
 *
 * Conventions (all arrays C-contiguous, little-endian):
 *   samples  int8   [C][P+2][F][Tp][Rpp][Pol=2][2]      (LambdaConfig::InputPacketSamplesType)
 *   scales   int16  [C][P+2][R][Pol]                    (LambdaConfig::PacketScalesType)
 *   weights  fp16   [C][Pol][B][R][2]                   (BeamWeightsT<T>)
 *   gains    float  [C][Pol][R][2]                      (LambdaConfig::AntennaGains)
 *   vis      int32  [C][R(R+1)/2][Pol][Pol][2]          baseline(i,j)=j(j+1)/2+i, i<=j,
 *                                                        value sum_t x_{i,p} conj(x_{j,q})
 *   evals    float  [batch][R] ascending;  evecs float2 [batch][R(k)][R(l)] (component l of
 *                                                        eigenvector k)
 *   beams    fp16   [C][Pol][NB][T][2]                  (LambdaConfig::BeamOutputType)
 *   spectra  float  [C][Pol][NB][bins]                  (FFTOutputType of each pipeline)
 * where R = F * Rpp receivers, T = P * Tp samples per integration.
 *
 * Every entry point is asynchronous on the given stream, never synchronises
 * (except sf_plan_status, which says so), and returns an sf_status code.
 * The CUDA stream argument is a cudaStream_t passed as void*.
 */
#ifndef SF_CAPI_H
#define SF_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sf_status {
  SF_OK = 0,
  SF_ERR_INVALID_ARGUMENT = 1, /* bad shape, null pointer, out-of-range value */
  SF_ERR_UNSUPPORTED = 2,      /* shape outside what the kernels implement */
  SF_ERR_CUDA = 3,             /* a CUDA runtime call failed (sf_last_error has it) */
  SF_ERR_DEVICE = 4,           /* a kernel reported an error bit (sf_plan_status) */
  SF_ERR_NO_DEVICE = 5         /* no usable sm_103a device */
} sf_status;

/* Device error bits, OR-ed into a plan's status word (sf_plan_status) or the
 * caller's status word (sf_run_adaptive_noalloc). */
typedef enum sf_device_bits {
  SF_DEV_TIMEOUT_TMA = 1 << 0,       /* a packet copy never landed (bounded wait ran out) */
  SF_DEV_TIMEOUT_CONVERT = 1 << 1,   /* an operand-tile hand-off wait ran out */
  SF_DEV_TIMEOUT_MMA = 1 << 2,       /* a tensor-core wait ran out */
  SF_DEV_TIMEOUT_EPILOGUE = 1 << 3,  /* an accumulator drain wait ran out */
  SF_DEV_EIG_NOT_CONVERGED = 1 << 4, /* an eigensolver hit its sweep limit */
  SF_DEV_BAD_SHAPE = 1 << 5,         /* a kernel met a shape it does not implement */
  SF_DEV_BAD_DELAY = 1 << 6          /* a sub-packet delay outside [-Tp, Tp] was replaced by 0 */
} sf_device_bits;

/* Integration window inside the (P+2)-packet buffer. */
typedef enum sf_window {
  /* packets 0..P-1, no delay: LambdaCorrBeamOnlyGPUPipeline
     (reference include/spatial/spatial.cuh:215-304) */
  SF_WINDOW_PACKET = 0,
  /* starts one packet in, shifted per FPGA by the sub-packet delay:
     LambdaGPUPipeline / adaptive (reference include/spatial/spatial.cuh:1420-1506) */
  SF_WINDOW_ALIGNED = 1
} sf_window;

/* Which covariance blocks are eigendecomposed. */
typedef enum sf_eig_mode {
  /* all Pol x Pol blocks, no whitening: batch C*Pol*Pol
     (reference include/spatial/pipeline/lambda_gpu_pipeline.hpp:438-439, 494-501) */
  SF_EIG_ALL_BLOCKS = 0,
  /* same-polarisation blocks with diagonal whitening: batch C*Pol
     (reference lambda_adaptive_beamformed_spectra_pipeline.hpp:648-686) */
  SF_EIG_SAME_POL_WHITENED = 1
} sf_eig_mode;

/* How the number K of nulled modes is chosen per (channel, pol). */
typedef enum sf_k_rule {
  SF_K_FIXED = 0,       /* per-channel counts from sf_set_fixed_counts (default 0) */
  SF_K_DETECT = 1,      /* K = #{lambda > p50 + delta (p80-p20)/1.6832}
                           (reference include/spatial/spatial.cuh:900-950) */
  SF_K_NOISE_FLOOR = 2  /* K = #{lambda > delta x median(lambda)} */
} sf_k_rule;

typedef struct sf_shape {
  int32_t n_channels;             /* C */
  int32_t n_fpgas;                /* F */
  int32_t n_time_per_packet;      /* Tp */
  int32_t n_receivers;            /* R = F * Rpp */
  int32_t n_polarizations;        /* must be 2 */
  int32_t n_receivers_per_packet; /* Rpp */
  int32_t n_packets;              /* P packets per integration */
  int32_t n_beams;                /* B */
} sf_shape;

typedef struct sf_plan sf_plan;

/* Plan lifetime.  Replaces the constructors of LambdaGPUPipeline /
 * LambdaCorrBeamOnlyGPUPipeline / LambdaAdaptiveBeamformedSpectraPipeline
 * (reference include/spatial/pipeline/lambda_gpu_pipeline.hpp:784-797,
 * lambda_corr_beam_only_gpu_pipeline.hpp:385-403,
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:1014-1036): allocates the
 * plan's device state on the current device. */
int sf_plan_create(const sf_shape *shape, sf_plan **out_plan);
int sf_plan_destroy(sf_plan *plan);
int sf_plan_get_shape(const sf_plan *plan, sf_shape *out_shape);

/* Text of the last error on the calling thread (never NULL). */
const char *sf_last_error(void);

/* Reads and clears the plan's device error bits; synchronises `stream`.
 * Replaces the reference's unread cuSOLVER info / CUDA_CHECK exits
 * (reference include/spatial/logging.hpp:11-50). */
int sf_plan_status(sf_plan *plan, void *stream, uint32_t *out_bits);

/* ---- configuration (host arrays copied into plan device memory) ---------- */

/* GPUPipeline::set_subpacket_delays (reference include/spatial/pipeline_base.hpp:15-17):
 * one delay per FPGA in samples, each in [-Tp, Tp]; NULL resets to zero. */
int sf_set_subpacket_delays(sf_plan *plan, const int32_t *h_delays, void *stream);

/* GPUPipeline::set_antenna_gains (pipeline_base.hpp:18-20): complex gains
 * [C][Pol][R][2] floats; NULL resets to 1. */
int sf_set_antenna_gains(sf_plan *plan, const float *h_gains, void *stream);

/* GPUPipeline::set_fine_delays (pipeline_base.hpp:21-22): per-receiver delays
 * in ns folded into the weights as exp(-2 pi i f_c tau), f_c = base + (min_ch + c) bw. */
int sf_set_fine_delays(sf_plan *plan, const float *h_delays_ns, double base_freq_hz,
                       double channel_bw_hz, int32_t min_freq_ch, void *stream);

/* GPUPipeline::set_stream_permutation (reference include/spatial/pipeline/lambda_gpu_pipeline.hpp:1139-1150,
 * reorder_streams_kernel spatial.cuh:596-636): canonical output stream k = 2 r + p (receiver r,
 * pol p) takes source receiver h_recv_perm[k] (flat f * Rpp + n, packet order) at source pol
 * h_pol_perm[k]; h_recv_perm[k] = -1 gives a zero stream.  Both arrays have 2R entries; both NULL
 * restores the identity.  Applied while the correlator/beamformer load their tiles (after the
 * window alignment, as the reference); gains stay with the source stream, fine-delay phasors with
 * the output receiver. */
int sf_set_stream_permutation(sf_plan *plan, const int32_t *h_recv_perm, const int32_t *h_pol_perm,
                              void *stream);

/* Beam weights, BeamWeightsT<T> payload (reference include/spatial/pipeline/common.hpp:52-55). */
int sf_set_weights(sf_plan *plan, const uint16_t *h_weights_f16, void *stream);

/* Steering-weight synthesis on the device, replacing compute_steering_weights and the weight copy of
 * BeamSteering::maybe_refresh (reference include/spatial/pipeline/common.hpp:97-185, 255-300): sets the
 * plan's weights (the payload sf_set_weights sets) to
 *   w[c][pol][b][r] = (1/R) G[c][pol][r] exp(i phase),  phase = -2 pi f_c / c_light (l e + m n + n u),
 *   f_c = base_freq_hz + (min_freq_ch + c) channel_bw_hz,
 * in double precision, rounded to float and then fp16 (as the reference); null inputs get exactly 0.
 *   h_dircos     double [B][3]        direction cosines (l, m, n) of each beam's target, local ENU frame
 *   h_enu        double [R][3]        position (east, north, up; metres) of each receiver's antenna
 *   h_connected  int32  [R]           0 = null input (no antenna on the stream); NULL = all connected
 *   h_cal_gains  float  [C][Pol][R][2] calibration gains G, or NULL for 1
 * Asynchronous, like the reference's refresh ("no GPU sync"): the host arrays are staged in the plan's
 * pinned memory before return (they are free on return) and the synthesis runs on `stream`, so runs
 * queued earlier on that stream finish on the old weights and later runs read the new ones.  A call
 * waits only for the previous call's staging copies to have landed, never for queued runs. */
int sf_set_steering_weights(sf_plan *plan, const double *h_dircos, const double *h_enu, const int32_t *h_connected,
                            double base_freq_hz, double channel_bw_hz, int32_t min_freq_ch, const float *h_cal_gains,
                            void *stream);

/* Device address of the plan's beam weights, laid out as the BeamWeightsT<T> payload
 * (fp16 pairs [C][Pol][B][R][2]), for a host steering object that enqueues its own
 * asynchronous copies into it on the plan's stream: the reference's
 * BeamSteering<T>::register_buffer(device_weights, stream) (reference
 * include/spatial/pipeline/common.hpp:245-250, 296-303).  Valid until sf_plan_destroy. */
int sf_plan_weights_buffer(sf_plan *plan, void **out_device_weights);

/* Fixed K per channel (the -e map of the adaptive pipeline,
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:1160-1167); NULL resets to 0. */
int sf_set_fixed_counts(sf_plan *plan, const int32_t *h_counts, void *stream);

/* ---- stage kernels --------------------------------------------------------- */

/* Correlate one integration into exact int32 visibilities on the tensor cores.
 * Replaces packet_to_corr_input / aligned_to_corr_input + tcc::Correlator +
 * corr_to_trimmed (reference spatial.cuh:55-304, lambda_gpu_pipeline.hpp:640-671,
 * src/spatial.cu:176-200). */
int sf_correlate(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                 int32_t window, int32_t *d_vis, void *stream);

/* Covariance + eigendecomposition + K + projection + effective weights for
 * each (channel, pol[, pol]) matrix.  Replaces unpack_triangular_baseline_batch,
 * diagonalWhiten, cusolverDnXsyevBatched, detectSignalEigenmodeCounts,
 * unwhitenEigenvectors, buildIdentityMinusProjection / shrink, and the ccglib
 * weight projection (reference spatial.cuh:672-713, 900-1148;
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:648-794).
 *   d_evals  [batch][R], d_evecs float2 [batch][R][R] (either may be NULL)
 *   d_counts int32 [C][Pol] (SAME_POL mode only; may be NULL)
 *   d_proj_f16 fp16 pairs [C][Pol][R][R] column-major projector (may be NULL)
 * In SAME_POL mode the effective weights for sf_beamform (2B beams: original,
 * projected) are left in plan memory. */
int sf_covariance_eig(sf_plan *plan, const int32_t *d_vis, int32_t eig_mode, int32_t k_rule,
                      float delta, int32_t shrink, float *d_evals, float *d_evecs,
                      int32_t *d_counts, uint16_t *d_proj_f16, void *stream);

/* The effective weights the last sf_covariance_eig in SAME_POL mode (or sf_run_adaptive) left in
 * plan memory -- the pair sf_beamform applies -- copied into d_weff: float pairs [C][Pol][2B][R][2],
 * slot 0 (rows 0..B-1) = W diag(d), slot 1 (rows B..2B-1) = (W P) diag(d).  The reference keeps the
 * same pair in device memory only (weights_rfi_mitigated, slots 0 and 1,
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:764-790); this reads it out, e.g. to measure the
 * null depth |w'a|^2 / |w a|^2 on a known interferer.  Asynchronous device-to-device copy. */
int sf_get_effective_weights(sf_plan *plan, float *d_weff, void *stream);

/* Beamform with the plan's effective weights: n_slots = 1 uses W diag(d),
 * n_slots = 2 uses the (original, projected) pair from sf_covariance_eig.
 * Replaces aligned_to_col_maj_cons + weights permutation + ccglib GEMM +
 * beam_ccglib_to_half_output (reference spatial.cuh:145-213, 376-418;
 * lambda_gpu_pipeline.hpp:708-743). */
int sf_beamform(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales, int32_t window,
                int32_t n_slots, uint16_t *d_beams_f16, void *stream);

/* Visibility integration across runs: accumulate int32 into int64
 * (reference src/spatial.cu:62-71, 126-170) and convert the accumulator to the
 * reference's float output with the gain/phasor factors applied
 * (VisibilitiesOutputType, packet_formats.hpp:351-353; dump_visibilities,
 * lambda_gpu_pipeline.hpp:1153-1194). */
int sf_accumulate_visibilities(sf_plan *plan, const int32_t *d_vis, int64_t *d_accum,
                               void *stream);
int sf_visibilities_to_float(sf_plan *plan, const int64_t *d_accum, float *d_vis_f32,
                             void *stream);

/* ---- beam spectra ------------------------------------------------------------ */

/* LambdaGPUPipeline's spectra tail (reference lambda_gpu_pipeline.hpp:522-531 with the cuFFT plan
 * of :814-817/:944-947, detect_and_downsample_fft spatial.cuh:795-848): per (channel, pol, beam)
 * a forward T-point FFT of the beam series (X[k] = sum_n x[n] exp(-2 pi i n k / T), fp32), then
 * bin g = mean of |X|^2 over bins g D .. g D + D - 1 with NaN bins skipped (0 if all NaN).
 *   d_beams_f16  fp16 pairs [C][Pol][n_beams_out][T][2] (sf_beamform's output)
 *   d_spectra    float [C][Pol][n_beams_out][T / downsample]  (FFTOutputType)
 * T = P * Tp must be a power of two in [64, 16384] (else SF_ERR_UNSUPPORTED). */
int sf_beam_spectra(sf_plan *plan, const uint16_t *d_beams_f16, int32_t n_beams_out,
                    int32_t downsample, float *d_spectra, void *stream);

/* The adaptive pipeline's spectra tail (reference lambda_adaptive_beamformed_spectra_pipeline.hpp:
 * 808-848, sum_fft_over_packets spatial.cuh:1508-1567): per (channel, pol, beam) and packet a
 * Tp-point forward FFT, bins kept in the order Tp/2+trim .. Tp-1, 0 .. Tp/2-trim-1 (the reference
 * uses trim = 5, NR_FINE_CHANNELS_TO_REMOVE_EACH_SIDE), |X| summed over the P packets.
 *   d_beams_f16  fp16 pairs [C][Pol][n_beams_out][T][2], 16-byte aligned
 *   d_spectra    float [C][Pol][n_beams_out][Tp - 2 trim]
 * Tp must be 16, 32 or 64 (the reference's plan is fixed at 64). */
int sf_packet_spectra(sf_plan *plan, const uint16_t *d_beams_f16, int32_t n_beams_out, int32_t trim,
                      float *d_spectra, void *stream);

/* ---- whole chains (what the drop-in pipelines run per buffer) -------------- */

/* LambdaCorrBeamOnlyGPUPipeline::enqueue_main (lambda_corr_beam_only_gpu_pipeline.hpp:305-344).
 * One pass over the samples yields visibilities and beams when the fused
 * tensor-memory layout fits (4R + the beam columns; not at R = 48) and
 * d_samples is 16-byte aligned; otherwise a correlation and a beamforming
 * launch give the same outputs.  The same holds for sf_run_lambda_gpu. */
int sf_run_corr_beam(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                     int32_t *d_vis, uint16_t *d_beams_f16, void *stream);

/* LambdaGPUPipeline::execute_pipeline compute (lambda_gpu_pipeline.hpp:445-531):
 * aligned window, all-blocks eigendecomposition, unprojected beams. */
int sf_run_lambda_gpu(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                      int32_t *d_vis, float *d_evals, float *d_evecs, uint16_t *d_beams_f16,
                      void *stream);

/* Adaptive null/shrink chain (lambda_adaptive_beamformed_spectra_pipeline.hpp:563-798):
 * corr -> whitened eig -> K -> I - U U^H (or shrink) -> W P -> 2B beams. */
int sf_run_adaptive(sf_plan *plan, const int8_t *d_samples, const int16_t *d_scales,
                    int32_t k_rule, float delta, int32_t shrink, int32_t *d_vis, float *d_evals,
                    float *d_evecs, int32_t *d_counts, uint16_t *d_beams_f16, void *stream);

/* ---- batched sub-arrays of uneven size --------------------------------------- */

/* A batch of units: one channel-integration each of a sub-array with its own receiver count
 * (a multiple of 4, at most 256; above 128 the refined precision path), all with n_samples (a
 * multiple of 128) samples and n_beams beams (at most 64; above 16 the refined path).
 * The whole mixed batch runs through one persistent tcgen05 correlator launch, the eigensolver
 * (one launch per size class, side by side on forked streams) and one persistent tcgen05
 * beamformer launch over a shared work list -- all capturable into one CUDA graph.  No counterpart
 * in the reference, which compiles one receiver count per build (LambdaConfig template parameters,
 * packet_formats.hpp:265-289) and replays one CUDA graph per buffer of that shape
 * (lambda_gpu_pipeline.hpp:1005-1046); per unit the chain is the adaptive pipeline's
 * (lambda_adaptive_beamformed_spectra_pipeline.hpp:563-798: corr -> whitened eig -> K ->
 * I - U U^H -> W P -> 2B beams) with unit receiver factors.
 *
 * Layout (offsets per unit from sf_batch_get_layout; units are grouped by receiver count):
 *   samples  int8  [T][R][Pol][2] at sample_off[u] bytes (the buffer 256-byte aligned)
 *   vis      int32 [R(R+1)/2][Pol][Pol][2] at vis_off[u]        (packed upper triangle)
 *   weights  fp16  [Pol][B][R][2] at weight_off[u] (fp16 pairs)
 *   evals    float [Pol][R] at eval_off[u] (whitened, ascending);  counts int32 [u][Pol]
 *   beams    fp16  [Pol][2B][T][2] at beam_off[u] (fp16 pairs; slot 0 original, slot 1 projected)
 * totals[5] = {sample bytes, vis elements, weight pairs, eval elements, beam pairs}. */
/* Beam operand precision of the batched beamformer (sf_batch_set_precision); accumulation is FP32. */
typedef enum sf_beam_precision {
  SF_BEAM_FP16 = 0,       /* fp16 samples (exact) and weights: the plain path */
  SF_BEAM_BF16 = 1,       /* bf16 samples (exact) and weights */
  SF_BEAM_E4M3 = 2,       /* e4m3 samples (rounded) and weights with per-beam scales (kind::f8f6f4) */
  SF_BEAM_E4M3_SPLIT = 3  /* e4m3 weights with per-beam scales, samples exact as 16 (x >> 4) + (x & 15) */
} sf_beam_precision;

typedef struct sf_batch sf_batch;
int sf_batch_create(int32_t n_units, const int32_t *h_receivers, int32_t n_samples, int32_t n_beams,
                    sf_batch **out_batch);
int sf_batch_destroy(sf_batch *batch);
int sf_batch_get_layout(const sf_batch *batch, int64_t *totals, int64_t *sample_off, int64_t *vis_off,
                        int64_t *weight_off, int64_t *eval_off, int64_t *beam_off);
/* Host weights in the layout above (all units); synchronises `stream`. */
int sf_batch_set_weights(sf_batch *batch, const uint16_t *h_weights_f16, void *stream);
/* K per unit for SF_K_FIXED (both pols); NULL resets to 0; synchronises `stream`. */
int sf_batch_set_fixed_counts(sf_batch *batch, const int32_t *h_counts, void *stream);
int sf_batch_correlate(sf_batch *batch, const int8_t *d_samples, int32_t *d_vis, void *stream);
int sf_batch_covariance_eig(sf_batch *batch, const int32_t *d_vis, int32_t k_rule, float delta, int32_t shrink,
                            float *d_evals, int32_t *d_counts, void *stream);
int sf_batch_beamform(sf_batch *batch, const int8_t *d_samples, uint16_t *d_beams_f16, void *stream);
/* The three stages; every call only enqueues work on `stream` (capturable). */
int sf_batch_run(sf_batch *batch, const int8_t *d_samples, int32_t k_rule, float delta, int32_t shrink,
                 int32_t *d_vis, float *d_evals, int32_t *d_counts, uint16_t *d_beams_f16, void *stream);
/* Reads and clears the batch's device error bits; synchronises `stream`. */
int sf_batch_status(sf_batch *batch, void *stream, uint32_t *out_bits);
/* The precision form: beam operands in `beam_precision` (sf_beam_precision), and -- with
 * refine_steps >= 0 -- the eigensolver's FP32 top-K vectors refined in FP64 (refine_steps subspace
 * steps, each A V, orthonormalisation and a Rayleigh-Ritz solve of V^H A V) before the weights are
 * projected in FP64, onto the orthogonal complement of an orthonormalised nulled subspace
 * (orthogonal != 0) or with the reference's I - U U^H of the un-whitened vectors (orthogonal = 0).
 * refine_steps = -1 keeps the FP32 top-K path (at most 128 receivers and 16 beams).  Units of more
 * than 128 receivers or batches of more than 16 beams always take the refined path; e4m3 beams need
 * it (it computes their per-beam scales: s = max |re w|, |im w| / 448, weights / s in e4m3, output
 * times s).  No counterpart in the reference (FP32 cuSOLVER vectors, fp16 projector and beams,
 * lambda_adaptive_beamformed_spectra_pipeline.hpp:679-798). */
int sf_batch_set_precision(sf_batch *batch, int32_t beam_precision, int32_t refine_steps, int32_t orthogonal);
/* The effective weights of the last eigen stage (what the beamformer applies), float pairs per unit
 * [Pol][2B][R][2] (slot 0 original, slot 1 projected) at weight_off[u] x 4 floats (the layout's weight
 * offsets, doubled for the two slots).  Asynchronous device-to-device copy. */
int sf_batch_effective_weights(sf_batch *batch, float *d_weff, void *stream);
/* After a refined run: per (unit, pol) the relative residual max_k ||A v_k - theta_k v_k|| / theta_max of
 * the FP32 vectors and of the refined ones (h_residuals [u][Pol][2], may be NULL) and the FP64 Ritz
 * values (h_ritz [u][Pol][8], descending, 0 past K; may be NULL).  Synchronises `stream`. */
int sf_batch_precision_report(sf_batch *batch, float *h_residuals, double *h_ritz, void *stream);
/* Times candidate work-list packings, ring depths and eigensolver concurrency on the given buffers
 * (CUDA events on `stream`, which it synchronises: call it at set-up, outside any capture), keeps
 * the fastest for later calls and writes a JSON record of every candidate and the choice into
 * `report` (if not NULL). */
int sf_batch_autotune(sf_batch *batch, const int8_t *d_samples, int32_t k_rule, float delta, int32_t *d_vis,
                      float *d_evals, int32_t *d_counts, uint16_t *d_beams_f16, void *stream, char *report,
                      int32_t report_len);

/* ---- learned subspace proposer -------------------------------------------------- */

/* A 3-layer MLP (in -> hidden -> hidden -> 8 n_receivers; ReLU after the hidden layers) mapping
 * one (channel, pol) whitened covariance to four complex start vectors of its interference
 * subspace, trained and run by hand-written BF16 tcgen05 GEMMs (fp32 accumulation, fp32 Adam
 * master weights).  Its features are the packed upper triangle of the whitened covariance
 * divided by its trace (2 x baselines real bf16 values, `in`; rows padded to in_ld).  No
 * counterpart in the reference, whose adaptive pipeline always runs the full eigensolve
 * (lambda_adaptive_beamformed_spectra_pipeline.hpp:679-686); that solve is the fallback here. */
typedef struct sf_proposer sf_proposer;
/* n_receivers in [8, 64]; hidden a multiple of 64; max_rows = the most covariances per call. */
int sf_proposer_create(int32_t n_receivers, int32_t hidden, int32_t max_rows, sf_proposer **out);
/* Synchronises the device, then frees. */
int sf_proposer_destroy(sf_proposer *proposer);
/* dims[6] = {in, in_ld, hidden, out, out_ld, max_rows}. */
int sf_proposer_dims(const sf_proposer *proposer, int32_t *dims);
/* Host fp32 parameters: layer l weight [out_l][in_l] (in_0 = in_ld) and bias [out_l]; resets the
 * Adam moments; synchronises `stream`.  get_params copies them back (NULL pointers skipped). */
int sf_proposer_set_params(sf_proposer *proposer, const float *w0, const float *b0, const float *w1,
                           const float *b1, const float *w2, const float *b2, void *stream);
int sf_proposer_get_params(const sf_proposer *proposer, float *w0, float *b0, float *w1, float *b1, float *w2,
                           float *b2, void *stream);
/* Features of every (channel, pol) covariance of `plan` from its visibilities: bf16 [2C][ldx]
 * (ldx >= in_ld; row c * 2 + p). */
int sf_proposer_features(const sf_plan *plan, const int32_t *d_vis, uint16_t *d_x, int32_t ldx, void *stream);
/* Training targets from a full eigendecomposition (sf_covariance_eig, SF_EIG_SAME_POL_WHITENED, with
 * eigenvalues and eigenvectors): the top four whitened eigenvectors, largest component real
 * positive, float [2C][4][R][2], and their weights clamp(1 - median / lambda_k, 0, 1) [2C][4]. */
int sf_proposer_targets(const sf_plan *plan, const int32_t *d_vis, const float *d_evals, const float *d_evecs,
                        float *d_targets, float *d_weights, void *stream);
/* Forward pass: d_y float [rows][out] (vector k of a row at k 2R, re/im interleaved). */
int sf_proposer_infer(sf_proposer *proposer, const uint16_t *d_x, int32_t rows, float *d_y, void *stream);
/* One Adam step on a batch: forward, phase-invariant weighted loss
 * sum_k w_k (|y_k|^2 + 1 - 2 |<t_k, y_k>|) / rows (added to *d_loss), backward, Adam (learning rate lr). */
int sf_proposer_train_step(sf_proposer *proposer, const uint16_t *d_x, const float *d_targets,
                           const float *d_weights, int32_t rows, float lr, float *d_loss, void *stream);
/* Reads and clears the proposer's device error bits; synchronises `stream`. */
int sf_proposer_status(sf_proposer *proposer, void *stream, uint32_t *out_bits);
/* The BF16 GEMM behind the proposer, exposed for tests: C[M][N] = sum_k A(m, k) B(n, k), A and B
 * bf16, K-major ([M][K] / [N][K]) or MN-major ([K][M] / [K][N]); epilogue 0: bf16 relu(acc + bias),
 * 1: fp32 acc + bias, 2: bf16 acc x [mask > 0], 3: fp32 out += acc (atomic; k_splits > 1 allowed).
 * Row pitches (elements) multiples of 8 and A, B 16-byte aligned; device error bits are OR-ed into
 * *d_status. */
int sf_gemm_bf16(int32_t M, int32_t N, int32_t K, const uint16_t *A, int32_t lda, int32_t a_mn_major,
                 const uint16_t *B, int32_t ldb, int32_t b_mn_major, int32_t epilogue, const float *bias,
                 const uint16_t *mask, int32_t ldm, void *out, int32_t ldo, int32_t k_splits, uint32_t *d_status,
                 void *stream);
/* The learned eigen stage in place of sf_covariance_eig (SF_EIG_SAME_POL_WHITENED): features ->
 * MLP -> n_iter subspace iterations U <- orth(A U) from its four start vectors -> Rayleigh-Ritz
 * (4 x 4 complex Jacobi) -> K (fixed, or theta > delta x noise floor with the floor
 * (tr A - sum theta) / (n - 4)) -> the plan's effective weights with I - U_K U_K^H.  A matrix
 * whose residual ||A u_k - theta_k u_k|| exceeds tol x theta_0, whose K exceeds 4, or whose rule
 * needs every eigenvalue (SF_K_DETECT) is listed on the device and solved by the full top-K
 * eigensolver instead, so it gets exactly the plain chain's weights.  d_ritz float [2C][4] and
 * d_fallback_count (one int32, the number of rejected matrices) may be NULL. */
int sf_covariance_eig_learned(sf_plan *plan, sf_proposer *proposer, const int32_t *d_vis, int32_t k_rule,
                              float delta, int32_t n_iter, float tol, int32_t *d_counts, float *d_ritz,
                              int32_t *d_fallback_count, void *stream);
/* correlate -> learned eigen stage -> beams (2B per pol), as sf_run_adaptive. */
int sf_run_adaptive_learned(sf_plan *plan, sf_proposer *proposer, const int8_t *d_samples,
                            const int16_t *d_scales, int32_t k_rule, float delta, int32_t n_iter, float tol,
                            int32_t *d_vis, int32_t *d_counts, uint16_t *d_beams_f16,
                            int32_t *d_fallback_count, void *stream);

/* ---- allocation-free variant ------------------------------------------------ */

/* The adaptive chain of sf_run_adaptive for callers that cannot allocate
 * device memory: code on a real-time thread or in a host callback that must
 * never block on the allocator, or a plugin whose host hands it pre-allocated
 * buffers and forbids cudaMalloc.  No counterpart in the reference (its
 * pipelines allocate their buffers in their constructors).
 *
 * Takes the shape and caller-owned device buffers only (no plan):
 *   d_weights_f16  fp16 pairs [C][Pol][B][R][2]
 *   d_factors      float pairs [C][Pol][R][2] per-receiver gain x phasor, or NULL for 1
 *   d_delays       int32 [F] sub-packet delays in [-Tp, Tp], or NULL for 0; a delay
 *                  outside that range is replaced by 0 and raises SF_DEV_BAD_DELAY
 *                  in the status word (the kernels never read outside the samples)
 *   d_fixed_counts int32 [C] K per channel for SF_K_FIXED, or NULL for 0
 *   d_counts       int32 [C][Pol] chosen K (may be NULL)
 *   d_beams_f16    fp16 [C][Pol][2B][T][2] (slot 0 original, slot 1 projected)
 *   d_status       uint32 device error bits (sf_device_bits); the call only ORs bits
 *                  in, so the caller clears it (may be NULL)
 * Pointer alignment: samples 16 bytes, factors 8 bytes, weights and beams 4 bytes
 * (else SF_ERR_INVALID_ARGUMENT).
 * Intermediates (visibilities, effective weights, ...) live in one 16 MiB
 * static device array per GPU, held from first use until the process exits;
 * shapes that need more (above about 530 channels of 36 receivers and 8 beams)
 * return SF_ERR_UNSUPPORTED.  The first call on each device is the set-up
 * call: it resolves the array's address (cudaGetSymbolAddress), which may load
 * the library's device code and commit the 16 MiB, so make it outside the
 * real-time path and before any stream capture; later calls allocate nothing.  Calls share the array and keep its last contents, so calls that
 * overlap on one GPU race: serialise them.  Allocates nothing (no cudaMalloc,
 * cudaFree or allocating library call). */
int sf_run_adaptive_noalloc(const sf_shape *shape, const int8_t *d_samples,
                            const int16_t *d_scales, const uint16_t *d_weights_f16,
                            const float *d_factors, const int32_t *d_delays,
                            const int32_t *d_fixed_counts, int32_t k_rule, float delta,
                            int32_t shrink, int32_t *d_counts, uint16_t *d_beams_f16,
                            uint32_t *d_status, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SF_CAPI_H */
