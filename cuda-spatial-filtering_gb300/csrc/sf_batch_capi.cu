// C ABI of the batched form over sub-arrays of uneven size (sf_capi.h,
// "batched sub-arrays"): batch lifetime and layout, the three stages over the
// whole mixed batch, and the autotuner that picks the work-list packing and
// ring depths of the correlator and beamformer and the concurrency of the
// eigensolver's size classes.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "sf_batch.cuh"
#include "sf_common.cuh"

int sf_internal_set_error(int code, const char *msg);
int sf_refine64_kmax();
cudaError_t sf_launch_refine64(const SfEigItem *items, int count, const int32_t *vis, const float2 *u32,
                               const int32_t *counts, const __half2 *weights, float2 *weff,
                               int B, int steps, int orthogonal, double *ritz, float *resid, uint32_t *status,
                               cudaStream_t stream);

namespace {

int fail(int code, const char *fmt, ...) {
  char buf[320];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return sf_internal_set_error(code, buf);
}

int cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaErrorInvalidConfiguration) return fail(SF_ERR_UNSUPPORTED, "%s: shape does not fit the kernel", what);
  return fail(SF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define BT_TRY(call, what)                       \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

constexpr int N_EIG_GROUPS = 3;  // eigensolver size classes: n <= 32, <= 64, <= 128
constexpr int MAX_R = 256;       // receivers per unit (above 128: the precision path)
constexpr int MAX_B_PRECISION = 64;
constexpr int MAX_NBG = 32;      // beams per pol (all slots) of one beamformer item

template <typename T> int upload(T **dst, const std::vector<T> &src) {
  if (*dst) cudaFree(*dst);
  *dst = nullptr;
  if (src.empty()) return SF_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dst), sizeof(T) * src.size());
  if (e == cudaSuccess) e = cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? SF_OK : cuda_fail(e, "batch upload");
}

}  // namespace

struct sf_batch {
  int n_units, T, B, num_sms;
  std::vector<int> R;
  std::vector<SfBatchUnit> units;
  std::vector<SfBatchItem> corr_items, beam_items;
  std::vector<long long> samp_off, vis_off, weight_off, eval_off, beam_off;
  long long samp_bytes = 0, vis_elems = 0, weight_elems = 0, eval_elems = 0, beam_elems = 0, weff_elems = 0;
  SfBatchLaunch L;
  SfBatchUnit *d_units = nullptr;
  SfBatchItem *d_corr_items = nullptr, *d_beam_items = nullptr;
  int *d_corr_first = nullptr, *d_corr_order = nullptr, *d_beam_first = nullptr, *d_beam_order = nullptr;
  // eigensolver: matrices grouped by size class
  std::vector<SfEigItem> eig_items;
  SfEigItem *d_eig_items = nullptr;
  int eig_first[N_EIG_GROUPS + 1] = {0, 0, 0, 0};
  int eig_nmax[N_EIG_GROUPS] = {0, 0, 0};
  bool eig_concurrent = true;
  cudaStream_t side[N_EIG_GROUPS] = {nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[N_EIG_GROUPS] = {nullptr, nullptr, nullptr};
  __half2 *d_weights = nullptr;
  float2 *d_weff = nullptr;
  int32_t *d_fixed = nullptr;
  uint32_t *d_status = nullptr;
  double corr_conv_weight = 32.0, beam_conv_weight = 32.0;
  std::string tuned;  // the autotuner's last choice (JSON)
  // precision path: FP32 top-K vectors, FP64 refinement + re-projection, bf16 / e4m3 beams
  bool precision = false;   // set by sf_batch_set_precision (forced for R > 128 or B > 16)
  bool needs_precision = false;
  int refine_steps = 2, orthogonal = 1;
  float2 *d_u = nullptr;         // FP32 vectors [item][min(n, 64)][n]
  float2 *d_gA = nullptr;        // working matrices of the n > 128 eigensolver, one per CTA
  int gA_grid = 0, n_max = 0;
  double *d_ritz = nullptr;
  float *d_resid = nullptr;
  float *d_scales = nullptr;
  int eig_small_count = 0;  // eig items with n <= 128 come first in the precision order
  std::vector<SfEigItem> peig_items;
  SfEigItem *d_peig_items = nullptr;
};

namespace {

void free_batch(sf_batch *b) {
  if (!b) return;
  cudaFree(b->d_units);
  cudaFree(b->d_corr_items);
  cudaFree(b->d_beam_items);
  cudaFree(b->d_corr_first);
  cudaFree(b->d_corr_order);
  cudaFree(b->d_beam_first);
  cudaFree(b->d_beam_order);
  cudaFree(b->d_eig_items);
  cudaFree(b->d_weights);
  cudaFree(b->d_weff);
  cudaFree(b->d_fixed);
  cudaFree(b->d_status);
  cudaFree(b->d_u);
  cudaFree(b->d_gA);
  cudaFree(b->d_ritz);
  cudaFree(b->d_resid);
  cudaFree(b->d_scales);
  cudaFree(b->d_peig_items);
  for (int g = 0; g < N_EIG_GROUPS; ++g) {
    if (b->side[g]) cudaStreamDestroy(b->side[g]);
    if (b->join[g]) cudaEventDestroy(b->join[g]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  delete b;
}

// (Re)builds the per-CTA work lists of both kernels for the current tuning.
int schedule(sf_batch *b) {
  std::vector<int> first, order;
  sf_batch_schedule(b->corr_items, b->units, b->T / 128, false, 4, 2 * b->B, b->L.corr_grid, b->corr_conv_weight,
                    first, order);
  if (int rc = upload(&b->d_corr_first, first)) return rc;
  if (int rc = upload(&b->d_corr_order, order)) return rc;
  sf_batch_schedule(b->beam_items, b->units, b->T / 128, true, b->L.beam_sa, 2 * b->B, b->L.beam_grid,
                    b->beam_conv_weight, first, order);
  if (int rc = upload(&b->d_beam_first, first)) return rc;
  if (int rc = upload(&b->d_beam_order, order)) return rc;
  b->L.d_corr_first = b->d_corr_first;
  b->L.d_corr_order = b->d_corr_order;
  b->L.d_beam_first = b->d_beam_first;
  b->L.d_beam_order = b->d_beam_order;
  return SF_OK;
}

int check(const sf_batch *b) { return b ? SF_OK : fail(SF_ERR_INVALID_ARGUMENT, "batch is NULL"); }

}  // namespace

extern "C" {

int sf_batch_create(int32_t n_units, const int32_t *h_receivers, int32_t n_samples, int32_t n_beams,
                    sf_batch **out) {
  if (!out || !h_receivers) return fail(SF_ERR_INVALID_ARGUMENT, "receivers / out is NULL");
  *out = nullptr;
  if (n_units < 1) return fail(SF_ERR_INVALID_ARGUMENT, "n_units must be >= 1");
  if (n_samples < 128 || n_samples % 128 != 0)
    return fail(SF_ERR_UNSUPPORTED, "n_samples must be a positive multiple of 128 (got %d)", n_samples);
  if (n_beams < 1 || n_beams > MAX_B_PRECISION)
    return fail(SF_ERR_UNSUPPORTED, "n_beams must be in [1, %d]", MAX_B_PRECISION);
  for (int u = 0; u < n_units; ++u)
    if (h_receivers[u] < 4 || h_receivers[u] % 4 != 0 || h_receivers[u] > MAX_R)
      return fail(SF_ERR_UNSUPPORTED, "unit %d: receivers must be a multiple of 4 in [4, %d] (got %d)", u, MAX_R,
                  h_receivers[u]);
  int dev = 0, major = 0, minor = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(SF_ERR_NO_DEVICE, "no CUDA device");
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (major != 10 || minor != 3) return fail(SF_ERR_NO_DEVICE, "this library is built for sm_103a");

  sf_batch *b = new (std::nothrow) sf_batch();
  if (!b) return fail(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  b->n_units = n_units;
  b->T = n_samples;
  b->B = n_beams;
  b->num_sms = sms;
  b->R.assign(h_receivers, h_receivers + n_units);
  memset(&b->L, 0, sizeof(b->L));
  b->L.T = n_samples;
  b->L.NB = 2 * n_beams;

  // size classes (ascending receiver count), each one contiguous sample array
  std::map<int, int> cls_of;
  for (int r : b->R) cls_of[r] = 0;
  if ((int)cls_of.size() > SF_BATCH_MAX_CLASSES) {
    free_batch(b);
    return fail(SF_ERR_UNSUPPORTED, "at most %d distinct receiver counts per batch", SF_BATCH_MAX_CLASSES);
  }
  int nc = 0;
  for (auto &kv : cls_of) {
    kv.second = nc;
    b->L.class_R[nc] = kv.first;
    ++nc;
  }
  b->L.n_classes = nc;
  std::vector<long long> class_units(nc, 0);
  for (int r : b->R) ++class_units[cls_of[r]];
  long long base = 0;
  for (int c = 0; c < nc; ++c) {
    b->L.class_base[c] = base;
    b->L.class_rows[c] = class_units[c] * n_samples;
    base += (class_units[c] * n_samples * 4 * b->L.class_R[c] + 255) / 256 * 256;
  }
  b->samp_bytes = base;
  std::vector<long long> seen(nc, 0);
  b->units.resize(n_units);
  b->samp_off.resize(n_units);
  b->vis_off.resize(n_units);
  b->weight_off.resize(n_units);
  b->eval_off.resize(n_units);
  b->beam_off.resize(n_units);
  int max_atoms = 0;
  for (int u = 0; u < n_units; ++u) max_atoms = std::max(max_atoms, (4 * b->R[u] + 63) / 64);
  // beams per beamformer item: the most whose fp16 weight tile (all the unit's atoms x
  // 4 x beams rows of 128 B) fits beside two rings of two slabs
  int nbg = std::min(2 * n_beams, MAX_NBG);
  while (nbg > 4 && sf_batch_smem_bytes(true, 2, 2, 2, static_cast<uint32_t>(max_atoms * (((4 * nbg + 15) / 16) * 16) * 128)) >
                        (size_t)sf_device_max_smem())
    nbg >>= 1;
  max_atoms = 0;
  for (int u = 0; u < n_units; ++u) {
    const int R = b->R[u], c = cls_of[R];
    SfBatchUnit &un = b->units[u];
    un.R = R;
    un.cls = c;
    un.row0 = seen[c] * n_samples;
    b->samp_off[u] = b->L.class_base[c] + seen[c] * (long long)n_samples * 4 * R;
    ++seen[c];
    b->vis_off[u] = b->vis_elems;
    un.vis_off = b->vis_elems;
    b->vis_elems += (long long)R * (R + 1) / 2 * 8;
    b->weight_off[u] = b->weight_elems;
    b->weight_elems += 2LL * n_beams * R;
    b->eval_off[u] = b->eval_elems;
    b->eval_elems += 2LL * R;
    un.weff_off = b->weff_elems;
    b->weff_elems += 2LL * 2 * n_beams * R;
    b->beam_off[u] = b->beam_elems;
    un.beam_off = b->beam_elems;
    b->beam_elems += 2LL * 2 * n_beams * n_samples;
    sf_batch_corr_items(u, R, b->corr_items);
    // beamformer items: groups of at most MAX_NBG beams (all slots) per pol
    const int NB = 2 * n_beams;
    for (int g0 = 0; g0 < NB; g0 += nbg) {
      SfBatchItem bi{};
      bi.unit = u;
      bi.natoms = (4 * R + 63) / 64;
      bi.c0 = g0;
      bi.n = std::min(nbg, NB - g0);
      b->beam_items.push_back(bi);
      max_atoms = std::max(max_atoms, bi.natoms);
    }
    b->n_max = std::max(b->n_max, R);
  }
  b->L.NBG = nbg;
  b->L.beam_op = SF_BEAM_FP16;
  b->needs_precision = b->n_max > sf_eig_topk_max_n() || n_beams > sf_eig_topk_max_b();
  b->precision = b->needs_precision;
  b->L.max_atoms = max_atoms;
  // eigensolver items grouped by size class
  const int limits[N_EIG_GROUPS] = {32, 64, 128};
  int lo = 0;
  for (int g = 0; g < N_EIG_GROUPS; ++g) {
    b->eig_first[g] = (int)b->eig_items.size();
    for (int u = 0; u < n_units; ++u) {
      const int R = b->R[u];
      if (R <= lo || R > limits[g]) continue;
      for (int p = 0; p < 2; ++p) {
        SfEigItem e{};
        e.vis_off = b->vis_off[u];
        e.factor_off = 0;
        e.weight_off = b->weight_off[u] + (long long)p * n_beams * R;
        e.weff_off = b->units[u].weff_off + (long long)p * 2 * n_beams * R;
        e.eval_off = b->eval_off[u] + (long long)p * R;
        e.n = R;
        e.pol = p;
        e.count_idx = 2 * u + p;
        e.unit = u;
        b->eig_items.push_back(e);
        b->eig_nmax[g] = std::max(b->eig_nmax[g], R);
      }
    }
    lo = limits[g];
  }
  b->eig_first[N_EIG_GROUPS] = (int)b->eig_items.size();
  // precision path: every (unit, pol), n <= 128 first, then the larger ones, each with room for
  // min(n, 64) FP32 eigenvectors
  {
    long long ucur = 0;
    for (int pass = 0; pass < 2; ++pass)
      for (int u = 0; u < n_units; ++u) {
        const int R = b->R[u];
        if ((pass == 0) != (R <= 128)) continue;
        for (int p = 0; p < 2; ++p) {
          SfEigItem e{};
          e.vis_off = b->vis_off[u];
          e.weight_off = b->weight_off[u] + (long long)p * n_beams * R;
          e.weff_off = b->units[u].weff_off + (long long)p * 2 * n_beams * R;
          e.eval_off = b->eval_off[u] + (long long)p * R;
          e.u_off = ucur;
          e.n = R;
          e.pol = p;
          e.count_idx = 2 * u + p;
          e.unit = u;
          b->peig_items.push_back(e);
          ucur += (long long)std::min(R, 64) * R;
        }
      }
    b->eig_small_count = 0;
    for (const SfEigItem &e : b->peig_items) b->eig_small_count += e.n <= 128;
    cudaError_t eu = cudaMalloc(&b->d_u, sizeof(float2) * std::max(1LL, ucur));
    if (eu != cudaSuccess) {
      free_batch(b);
      return cuda_fail(eu, "precision vectors");
    }
  }
  for (int g = 0; g < N_EIG_GROUPS; ++g)
    if (!b->needs_precision && b->eig_nmax[g] > 0 &&
        sf_eig_topk_items_smem(b->eig_nmax[g], n_beams) > (size_t)sf_device_max_smem()) {
      const int nm = b->eig_nmax[g];
      free_batch(b);
      return fail(SF_ERR_UNSUPPORTED, "%d receivers with %d beams exceed the eigensolver's shared memory", nm,
                  n_beams);
    }
  b->L.corr_grid = sms;
  b->L.beam_grid = sms;
  b->L.corr_ni = 2;
  b->L.corr_nf = 2;
  // deepest beamformer rings that fit beside the weight tile
  {
    const uint32_t wt = static_cast<uint32_t>(max_atoms * (((4 * nbg + 15) / 16) * 16) * 128);
    const int depth = sf_batch_smem_bytes(true, 2, 3, 3, wt) <= (size_t)sf_device_max_smem() ? 3 : 2;
    b->L.beam_sa = 2;
    b->L.beam_ni = depth;
    b->L.beam_nf = depth;
  }

  int rc = upload(&b->d_units, b->units);
  if (!rc) rc = upload(&b->d_corr_items, b->corr_items);
  if (!rc) rc = upload(&b->d_beam_items, b->beam_items);
  if (!rc) rc = upload(&b->d_eig_items, b->eig_items);
  if (!rc) rc = upload(&b->d_peig_items, b->peig_items);
  if (!rc) {
    const int np = (int)b->peig_items.size();
    cudaError_t ep = cudaMalloc(&b->d_ritz, sizeof(double) * np * sf_refine64_kmax());
    if (ep == cudaSuccess) ep = cudaMalloc(&b->d_resid, sizeof(float) * np * 2);
    if (ep == cudaSuccess) ep = cudaMalloc(&b->d_scales, sizeof(float) * n_units * 2 * 2 * n_beams);
    if (ep == cudaSuccess && b->n_max > 128) {
      b->gA_grid = std::min(sms, np - b->eig_small_count);
      ep = cudaMalloc(&b->d_gA, sizeof(float2) * (size_t)b->gA_grid * b->n_max * (b->n_max + 1));
    }
    if (ep != cudaSuccess) rc = cuda_fail(ep, "precision buffers");
    b->L.d_scales = b->d_scales;
  }
  if (!rc) {
    b->L.d_units = b->d_units;
    b->L.d_corr_items = b->d_corr_items;
    b->L.d_beam_items = b->d_beam_items;
    rc = schedule(b);
  }
  cudaError_t e = cudaSuccess;
  if (!rc) e = cudaMalloc(&b->d_weights, sizeof(__half2) * b->weight_elems);
  if (!rc && e == cudaSuccess) e = cudaMalloc(&b->d_weff, sizeof(float2) * b->weff_elems);
  if (!rc && e == cudaSuccess) e = cudaMalloc(&b->d_fixed, sizeof(int32_t) * 2 * n_units);
  if (!rc && e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(uint32_t));
  if (!rc && e == cudaSuccess) e = cudaMemset(b->d_weights, 0, sizeof(__half2) * b->weight_elems);
  if (!rc && e == cudaSuccess) e = cudaMemset(b->d_fixed, 0, sizeof(int32_t) * 2 * n_units);
  if (!rc && e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(uint32_t));
  for (int g = 0; !rc && e == cudaSuccess && g < N_EIG_GROUPS; ++g) {
    e = cudaStreamCreateWithFlags(&b->side[g], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming);
  }
  if (!rc && e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (!rc && e == cudaSuccess) e = cudaDeviceSynchronize();
  if (!rc && e != cudaSuccess) rc = cuda_fail(e, "batch create");
  if (rc) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return SF_OK;
}

int sf_batch_destroy(sf_batch *batch) {
  if (batch) cudaDeviceSynchronize();
  free_batch(batch);
  return SF_OK;
}

int sf_batch_get_layout(const sf_batch *b, int64_t *totals, int64_t *sample_off, int64_t *vis_off,
                        int64_t *weight_off, int64_t *eval_off, int64_t *beam_off) {
  if (int rc = check(b)) return rc;
  if (totals) {
    totals[0] = b->samp_bytes;
    totals[1] = b->vis_elems;
    totals[2] = b->weight_elems;
    totals[3] = b->eval_elems;
    totals[4] = b->beam_elems;
  }
  for (int u = 0; u < b->n_units; ++u) {
    if (sample_off) sample_off[u] = b->samp_off[u];
    if (vis_off) vis_off[u] = b->vis_off[u];
    if (weight_off) weight_off[u] = b->weight_off[u];
    if (eval_off) eval_off[u] = b->eval_off[u];
    if (beam_off) beam_off[u] = b->beam_off[u];
  }
  return SF_OK;
}

int sf_batch_set_weights(sf_batch *b, const uint16_t *h_weights, void *stream) {
  if (int rc = check(b)) return rc;
  if (!h_weights) return fail(SF_ERR_INVALID_ARGUMENT, "weights are NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BT_TRY(cudaMemcpyAsync(b->d_weights, h_weights, sizeof(__half2) * b->weight_elems, cudaMemcpyHostToDevice, s),
         "batch weights upload");
  BT_TRY(cudaStreamSynchronize(s), "batch weights upload");
  return SF_OK;
}

int sf_batch_set_fixed_counts(sf_batch *b, const int32_t *h_counts, void *stream) {
  if (int rc = check(b)) return rc;
  std::vector<int32_t> k(2 * b->n_units, 0);
  for (int u = 0; u < b->n_units; ++u) {
    const int v = h_counts ? h_counts[u] : 0;
    if (v < 0 || v > b->R[u]) return fail(SF_ERR_INVALID_ARGUMENT, "count %d of unit %d outside [0, %d]", v, u, b->R[u]);
    k[2 * u] = k[2 * u + 1] = v;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BT_TRY(cudaMemcpyAsync(b->d_fixed, k.data(), sizeof(int32_t) * k.size(), cudaMemcpyHostToDevice, s), "counts upload");
  BT_TRY(cudaStreamSynchronize(s), "counts upload");
  return SF_OK;
}

int sf_batch_correlate(sf_batch *b, const int8_t *d_samples, int32_t *d_vis, void *stream) {
  if (int rc = check(b)) return rc;
  if (!d_samples || !d_vis) return fail(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (reinterpret_cast<uintptr_t>(d_samples) % 256 != 0)
    return fail(SF_ERR_INVALID_ARGUMENT, "samples must be 256-byte aligned");
  BT_TRY(sf_batch_launch(b->L, false, d_samples, d_vis, nullptr, nullptr, b->d_status,
                         static_cast<cudaStream_t>(stream)),
         "batch correlate");
  return SF_OK;
}

int sf_batch_covariance_eig(sf_batch *b, const int32_t *d_vis, int32_t k_rule, float delta, int32_t shrink,
                            float *d_evals, int32_t *d_counts, void *stream) {
  if (int rc = check(b)) return rc;
  if (!d_vis) return fail(SF_ERR_INVALID_ARGUMENT, "vis is NULL");
  if (k_rule < SF_K_FIXED || k_rule > SF_K_NOISE_FLOOR) return fail(SF_ERR_INVALID_ARGUMENT, "unknown K rule");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->precision) {
    // FP32 top-K vectors (n <= 128 in shared memory, larger in global scratch), then the FP64
    // refinement and re-projection of the weights, then the e4m3 per-beam scales
    const int np = (int)b->peig_items.size();
    if (shrink) return fail(SF_ERR_UNSUPPORTED, "the precision path nulls (no shrink mode)");
    BT_TRY(sf_launch_eig_topk_vectors(b->d_peig_items, 0, b->eig_small_count, 128, d_vis, b->d_fixed, k_rule, delta,
                                      d_evals, d_counts, b->d_u, nullptr, 0, b->d_status, s),
           "precision eig");
    BT_TRY(sf_launch_eig_topk_vectors(b->d_peig_items, b->eig_small_count, np - b->eig_small_count, b->n_max, d_vis,
                                      b->d_fixed, k_rule, delta, d_evals, d_counts, b->d_u, b->d_gA, b->gA_grid,
                                      b->d_status, s),
           "precision eig (global working matrices)");
    if (!d_counts) return fail(SF_ERR_INVALID_ARGUMENT, "the precision path needs the counts buffer");
    BT_TRY(sf_launch_refine64(b->d_peig_items, np, d_vis, b->d_u, d_counts, b->d_weights, b->d_weff, b->B,
                              b->refine_steps, b->orthogonal, b->d_ritz, b->d_resid, b->d_status, s),
           "FP64 refinement");
    if (b->L.beam_op == SF_BEAM_E4M3 || b->L.beam_op == SF_BEAM_E4M3_SPLIT)
      BT_TRY(sf_batch_launch_scales(b->L, b->n_units, b->d_weff, b->d_scales, s), "beam scales");
    return SF_OK;
  }
  // size classes up to 128 receivers: sf_eig_small.cu (four or sixteen warps per matrix)
  auto launch = [&](int g, cudaStream_t st) {
    const int first = b->eig_first[g], count = b->eig_first[g + 1] - b->eig_first[g];
    if (sf_eig_small_items_supported(b->eig_nmax[g], b->B))
      return sf_launch_eig_small_items(b->d_eig_items, first, count, b->eig_nmax[g], b->B, d_vis, nullptr,
                                       b->d_weights, b->d_fixed, k_rule, delta, shrink ? 1 : 0, d_evals, d_counts,
                                       b->d_weff, b->d_status, b->num_sms, st);
    return sf_launch_eig_topk_items(b->d_eig_items, first, count, b->eig_nmax[g], b->B, d_vis, nullptr,
                                    b->d_weights, b->d_fixed, k_rule, delta, shrink ? 1 : 0, d_evals, d_counts,
                                    b->d_weff, b->d_status, st);
  };
  if (!b->eig_concurrent) {
    for (int g = 0; g < N_EIG_GROUPS; ++g) BT_TRY(launch(g, s), "batch eig");
    return SF_OK;
  }
  // size classes side by side (fork / join through events: capturable)
  BT_TRY(cudaEventRecord(b->fork, s), "batch eig fork");
  for (int g = 0; g < N_EIG_GROUPS; ++g) {
    BT_TRY(cudaStreamWaitEvent(b->side[g], b->fork, 0), "batch eig fork");
    BT_TRY(launch(g, b->side[g]), "batch eig");
    BT_TRY(cudaEventRecord(b->join[g], b->side[g]), "batch eig join");
    BT_TRY(cudaStreamWaitEvent(s, b->join[g], 0), "batch eig join");
  }
  return SF_OK;
}

int sf_batch_beamform(sf_batch *b, const int8_t *d_samples, uint16_t *d_beams_f16, void *stream) {
  if (int rc = check(b)) return rc;
  if (!d_samples || !d_beams_f16) return fail(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (reinterpret_cast<uintptr_t>(d_samples) % 256 != 0)
    return fail(SF_ERR_INVALID_ARGUMENT, "samples must be 256-byte aligned");
  BT_TRY(sf_batch_launch(b->L, true, d_samples, nullptr, b->d_weff, reinterpret_cast<__half2 *>(d_beams_f16),
                         b->d_status, static_cast<cudaStream_t>(stream)),
         "batch beamform");
  return SF_OK;
}

int sf_batch_run(sf_batch *b, const int8_t *d_samples, int32_t k_rule, float delta, int32_t shrink, int32_t *d_vis,
                 float *d_evals, int32_t *d_counts, uint16_t *d_beams_f16, void *stream) {
  if (int rc = sf_batch_correlate(b, d_samples, d_vis, stream)) return rc;
  if (int rc = sf_batch_covariance_eig(b, d_vis, k_rule, delta, shrink, d_evals, d_counts, stream)) return rc;
  return sf_batch_beamform(b, d_samples, d_beams_f16, stream);
}

int sf_batch_set_precision(sf_batch *b, int32_t beam_precision, int32_t refine_steps, int32_t orthogonal) {
  if (int rc = check(b)) return rc;
  if (beam_precision < SF_BEAM_FP16 || beam_precision > SF_BEAM_E4M3_SPLIT)
    return fail(SF_ERR_INVALID_ARGUMENT, "unknown beam precision %d", beam_precision);
  if (refine_steps < -1 || refine_steps > 8) return fail(SF_ERR_INVALID_ARGUMENT, "refine_steps outside [-1, 8]");
  if (refine_steps < 0 && b->needs_precision)
    return fail(SF_ERR_UNSUPPORTED, "more than 128 receivers or 16 beams need the FP64-refined path");
  if ((beam_precision == SF_BEAM_E4M3 || beam_precision == SF_BEAM_E4M3_SPLIT) && refine_steps < 0)
    return fail(SF_ERR_UNSUPPORTED, "e4m3 beams need the FP64-refined path (it computes the per-beam scales)");
  b->L.beam_op = beam_precision;
  b->precision = refine_steps >= 0;
  b->refine_steps = refine_steps < 0 ? 0 : refine_steps;
  b->orthogonal = orthogonal ? 1 : 0;
  // e4m3 atoms pair the int8 boxes: an even number per slab
  if ((beam_precision == SF_BEAM_E4M3 || beam_precision == SF_BEAM_E4M3_SPLIT) && (b->L.beam_sa & 1)) {
    b->L.beam_sa = 2;
    if (int rc = schedule(b)) return rc;
  }
  return SF_OK;
}

int sf_batch_effective_weights(sf_batch *b, float *d_weff, void *stream) {
  if (int rc = check(b)) return rc;
  if (!d_weff) return fail(SF_ERR_INVALID_ARGUMENT, "weff is NULL");
  BT_TRY(cudaMemcpyAsync(d_weff, b->d_weff, sizeof(float2) * b->weff_elems, cudaMemcpyDeviceToDevice,
                         static_cast<cudaStream_t>(stream)),
         "effective weights copy");
  return SF_OK;
}

int sf_batch_precision_report(sf_batch *b, float *h_residuals, double *h_ritz, void *stream) {
  if (int rc = check(b)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t np = b->peig_items.size();
  // host copies are [unit][Pol] ordered: map from the precision item order
  std::vector<float> r(np * 2);
  std::vector<double> t(np * sf_refine64_kmax());
  BT_TRY(cudaMemcpyAsync(r.data(), b->d_resid, sizeof(float) * r.size(), cudaMemcpyDeviceToHost, s), "report");
  BT_TRY(cudaMemcpyAsync(t.data(), b->d_ritz, sizeof(double) * t.size(), cudaMemcpyDeviceToHost, s), "report");
  BT_TRY(cudaStreamSynchronize(s), "report");
  const int km = sf_refine64_kmax();
  for (size_t i = 0; i < np; ++i) {
    const int idx = b->peig_items[i].count_idx;
    if (h_residuals) {
      h_residuals[2 * idx] = r[2 * i];
      h_residuals[2 * idx + 1] = r[2 * i + 1];
    }
    if (h_ritz)
      for (int k = 0; k < km; ++k) h_ritz[(size_t)idx * km + k] = t[i * km + k];
  }
  return SF_OK;
}

int sf_batch_status(sf_batch *b, void *stream, uint32_t *out_bits) {
  if (int rc = check(b)) return rc;
  uint32_t bits = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BT_TRY(cudaMemcpyAsync(&bits, b->d_status, sizeof(bits), cudaMemcpyDeviceToHost, s), "batch status");
  BT_TRY(cudaMemsetAsync(b->d_status, 0, sizeof(uint32_t), s), "batch status");
  BT_TRY(cudaStreamSynchronize(s), "batch status");
  if (out_bits) *out_bits = bits;
  if (bits) return fail(SF_ERR_DEVICE, "device error bits 0x%x", bits);
  return SF_OK;
}

int sf_batch_autotune(sf_batch *b, const int8_t *d_samples, int32_t k_rule, float delta, int32_t *d_vis,
                      float *d_evals, int32_t *d_counts, uint16_t *d_beams_f16, void *stream, char *report,
                      int32_t report_len) {
  if (int rc = check(b)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  BT_TRY(cudaEventCreate(&e0), "autotune event");
  BT_TRY(cudaEventCreate(&e1), "autotune event");
  auto time_it = [&](auto &&fn, float &ms) -> int {
    for (int w = 0; w < 2; ++w)
      if (int rc = fn()) return rc;
    BT_TRY(cudaEventRecord(e0, s), "autotune");
    for (int r = 0; r < 3; ++r)
      if (int rc = fn()) return rc;
    BT_TRY(cudaEventRecord(e1, s), "autotune");
    BT_TRY(cudaEventSynchronize(e1), "autotune");
    BT_TRY(cudaEventElapsedTime(&ms, e0, e1), "autotune");
    ms /= 3.0f;
    return SF_OK;
  };
  std::string rep = "{\"corr\": [";
  // correlator: cost-model weight of the int8 -> fp16 conversion, ring depths
  const double conv_w[3] = {0.0, 32.0, 128.0};
  const int rings[2][2] = {{2, 2}, {3, 2}};
  float best = 1e30f;
  double best_w = b->corr_conv_weight;
  int best_r = 0;
  char buf[256];
  for (double w : conv_w)
    for (int r = 0; r < 2; ++r) {
      b->corr_conv_weight = w;
      b->L.corr_ni = rings[r][0];
      b->L.corr_nf = rings[r][1];
      if (sf_batch_smem_bytes(false, 4, b->L.corr_ni, b->L.corr_nf, 0) > (size_t)sf_device_max_smem()) continue;
      if (int rc = schedule(b)) return rc;
      float ms = 0;
      if (int rc = time_it([&] { return sf_batch_correlate(b, d_samples, d_vis, stream); }, ms)) return rc;
      snprintf(buf, sizeof(buf), "%s{\"conv_weight\": %.0f, \"ring\": [%d, %d], \"ms\": %.4f}",
               rep.back() == '[' ? "" : ", ", w, rings[r][0], rings[r][1], ms);
      rep += buf;
      if (ms < best) {
        best = ms;
        best_w = w;
        best_r = r;
      }
    }
  b->corr_conv_weight = best_w;
  b->L.corr_ni = rings[best_r][0];
  b->L.corr_nf = rings[best_r][1];
  snprintf(buf, sizeof(buf), "], \"corr_choice\": {\"conv_weight\": %.0f, \"ring\": [%d, %d], \"ms\": %.4f}",
           best_w, rings[best_r][0], rings[best_r][1], best);
  rep += buf;
  // eigensolver: size classes concurrent or one after another
  rep += ", \"eig\": [";
  float eb = 1e30f;
  bool best_conc = true;
  for (int conc = 1; conc >= 0; --conc) {
    b->eig_concurrent = conc != 0;
    float ms = 0;
    if (int rc = time_it([&] { return sf_batch_covariance_eig(b, d_vis, k_rule, delta, 0, d_evals, d_counts, stream); },
                         ms))
      return rc;
    snprintf(buf, sizeof(buf), "%s{\"concurrent\": %s, \"ms\": %.4f}", conc ? "" : ", ", conc ? "true" : "false", ms);
    rep += buf;
    if (ms < eb) {
      eb = ms;
      best_conc = conc != 0;
    }
  }
  b->eig_concurrent = best_conc;
  // beamformer: atoms per slab and ring depths
  rep += "], \"beam\": [";
  const int cand[4][3] = {{2, 3, 3}, {2, 2, 2}, {4, 1, 2}, {1, 4, 4}};
  float bb = 1e30f;
  int bc = 0;
  for (int c = 0; c < 4; ++c) {
    b->L.beam_sa = cand[c][0];
    b->L.beam_ni = cand[c][1];
    b->L.beam_nf = cand[c][2];
    const uint32_t wt = static_cast<uint32_t>(b->L.max_atoms * (((4 * 2 * b->B + 15) / 16) * 16) * 128);
    if (sf_batch_smem_bytes(true, cand[c][0], cand[c][1], cand[c][2], wt) > (size_t)sf_device_max_smem()) continue;
    if (int rc = schedule(b)) return rc;
    float ms = 0;
    if (int rc = time_it([&] { return sf_batch_beamform(b, d_samples, d_beams_f16, stream); }, ms)) return rc;
    snprintf(buf, sizeof(buf), "%s{\"atoms_per_slab\": %d, \"ring\": [%d, %d], \"ms\": %.4f}",
             rep.back() == '[' ? "" : ", ", cand[c][0], cand[c][1], cand[c][2], ms);
    rep += buf;
    if (ms < bb) {
      bb = ms;
      bc = c;
    }
  }
  b->L.beam_sa = cand[bc][0];
  b->L.beam_ni = cand[bc][1];
  b->L.beam_nf = cand[bc][2];
  if (int rc = schedule(b)) return rc;
  snprintf(buf, sizeof(buf),
           "], \"choice\": {\"corr_conv_weight\": %.0f, \"corr_ring\": [%d, %d], \"eig_concurrent\": %s, "
           "\"beam_atoms_per_slab\": %d, \"beam_ring\": [%d, %d]}, \"ms\": {\"corr\": %.4f, \"eig\": %.4f, "
           "\"beam\": %.4f}}",
           b->corr_conv_weight, b->L.corr_ni, b->L.corr_nf, b->eig_concurrent ? "true" : "false", b->L.beam_sa,
           b->L.beam_ni, b->L.beam_nf, best, eb, bb);
  rep += buf;
  b->tuned = rep;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (report && report_len > 0) {
    strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return SF_OK;
}

}  // extern "C"
