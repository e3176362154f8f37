// knn_api.cu -- C ABI entry points of the kNN pipelines: argument checks,
// the reference's k clamping, host<->device staging and timing.
#include <chrono>
#include <cmath>
#include <vector>

#include "knn_common.cuh"

namespace {

struct HostTimer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

}  // namespace

// Diagnostic outputs requested by the mds_knn_rms_screen / _superpose entry points.
struct KnnRmsHooks {
  uint64_t* screen_keys = nullptr;
  int* screen_counts = nullptr;
  int screen_kprime = 0;
  float* prep_dev = nullptr;
  float* prep_rec = nullptr;
};

static int knn_rms_impl(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz, int n_fit,
                        int natoms, const float* mass, int k, unsigned flags, double* out_d, int32_t* out_i,
                        int* k_used, const KnnRmsHooks& hooks);

extern "C" int mds_knn_rms(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz,
                           int n_fit, int natoms, const float* mass, int k, unsigned flags,
                           double* out_d, int32_t* out_i, int* k_used) {
  if (!ctx) return MDS_ERR_ARG;
  if (!out_d || !out_i) return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  return knn_rms_impl(ctx, ref_xyz, n_ref, fit_xyz, n_fit, natoms, mass, k, flags, out_d, out_i, k_used,
                      KnnRmsHooks{});
}

extern "C" int mds_knn_rms_screen(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz,
                                  int n_fit, int natoms, const float* mass, int kprime, unsigned flags,
                                  uint64_t* keys, int32_t* counts) {
  if (!ctx) return MDS_ERR_ARG;
  if (!keys || !counts || kprime < 1) return mds_fail(ctx, MDS_ERR_ARG, "keys/counts/kprime");
  if (flags & (MDS_DEVICE_IO | MDS_FULL))
    return mds_fail(ctx, MDS_ERR_ARG, "the screen diagnostic takes host buffers and a sorted run");
  KnnRmsHooks h;
  h.screen_keys = keys;
  h.screen_counts = counts;
  h.screen_kprime = kprime;
  return knn_rms_impl(ctx, ref_xyz, n_ref, fit_xyz, n_fit, natoms, mass, std::max(1, kprime / 2), flags,
                      nullptr, nullptr, nullptr, h);
}

extern "C" int mds_knn_rms_superpose(mds_ctx* ctx, const float* ref_xyz, int n_ref, int natoms,
                                     const float* mass, unsigned flags, float* dev, float* rec) {
  if (!ctx) return MDS_ERR_ARG;
  if (!dev || !rec) return mds_fail(ctx, MDS_ERR_ARG, "null output");
  if (flags & (MDS_DEVICE_IO | MDS_FULL)) return mds_fail(ctx, MDS_ERR_ARG, "host buffers, sorted run only");
  KnnRmsHooks h;
  h.prep_dev = dev;
  h.prep_rec = rec;
  double d = 0;
  int32_t i = 0;
  return knn_rms_impl(ctx, ref_xyz, n_ref, nullptr, 0, natoms, mass, 1, flags & ~MDS_PREC_MASK, &d, &i,
                      nullptr, h);
}

static int knn_rms_impl(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz, int n_fit,
                        int natoms, const float* mass, int k, unsigned flags, double* out_d, int32_t* out_i,
                        int* k_used, const KnnRmsHooks& hooks) {
  HostTimer timer;
  ctx->stats = mds_knn_stats{};
  if (!ref_xyz || !mass) return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  if (n_ref < 1 || natoms < 1 || n_fit < 0)
    return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes: n_ref=%d n_fit=%d natoms=%d", n_ref, n_fit, natoms);
  if (natoms > 16384)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "natoms=%d exceeds the supported maximum of 16384", natoms);
  const bool full = (flags & MDS_FULL) != 0;
  const bool dev = (flags & MDS_DEVICE_IO) != 0;
  const unsigned prec = flags & MDS_PREC_MASK;
  if (prec != MDS_PREC_FP32 && prec != MDS_PREC_BF16X3 && prec != MDS_PREC_FP16X3)
    return mds_fail(ctx, MDS_ERR_ARG, "unknown precision flag 0x%x", prec);
  if (!fit_xyz) n_fit = n_ref;
  // knn_rms.cpp:224-225: k is clamped to N_ref - 1 (k1 is taken as k + 1 of
  // the clamped k; the reference's stale k1 is undefined behaviour there).
  if (!full) {
    if (k < 0) return mds_fail(ctx, MDS_ERR_ARG, "k must be >= 0");
    if (n_ref - 1 < k) k = n_ref - 1;
    if (k + 1 > 416)
      return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d exceeds the supported maximum of 415", k);
  }
  if (k_used) *k_used = k;
  cudaSetDevice(ctx->device);
  KnnRmsPlan pl;
  pl.nref = n_ref;
  pl.nfit = n_fit;
  pl.natoms = natoms;
  pl.Ap = mds_round_up(natoms, 64);
  pl.k = k;
  pl.nofit = (flags & MDS_NOFIT) ? 1 : 0;
  pl.full = full ? 1 : 0;
  pl.noskip = (flags & MDS_NO_SKIP) ? 1 : 0;
  pl.prec = prec;
  // K' = 2(k+1) (at least k+33): the recheck stops early once the k+1 best
  // are settled, so a wide K' mainly makes the guard hold on the first pass
  // where neighbours crowd within the guard of one another. The tensor-core
  // screen's thresholds also follow the (k+1)-th bound, so a wide K' does not
  // loosen its tile skipping: there K' is 4(k+1) up to 256.
  const int kpmax = (prec == MDS_PREC_FP32) ? 448 : 352;
  pl.kprime = std::min(mds_round_up(tc_kprime_want(k, prec != MDS_PREC_FP32), 32), kpmax);
  if (!full && pl.kprime < k + 1 + 16)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d is too large for the %s screen (use fp32 precision)", k,
                    prec == MDS_PREC_FP32 ? "fp32" : "tensor-core");
  if (hooks.screen_keys) {
    if (hooks.screen_kprime > 448) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "kprime > 448");
    pl.kprime = hooks.screen_kprime;
    pl.screen_keys = hooks.screen_keys;
    pl.screen_counts = hooks.screen_counts;
  }
  pl.prep_dev = hooks.prep_dev;
  pl.prep_rec = hooks.prep_rec;
  pl.guard_fp32 = MDS_GUARD_FP32;
  pl.guard_tc = MDS_GUARD_TC;
  ctx->stats.pairs = (long long)n_ref * n_fit;
  ctx->stats.kprime = pl.kprime;
  if (n_fit == 0 || (!full && k == 0)) return MDS_OK;

  cudaStream_t s = ctx->stream;
  const size_t width = full ? (size_t)n_ref : (size_t)k;
  DevBuf dref(ctx), dfit(ctx), dd(ctx), di(ctx);
  const float* pref = ref_xyz;
  const float* pfit = fit_xyz;
  double* pd = out_d;
  int* pi = out_i;
  std::vector<float> hmass(natoms);
  if (!dev) {
    // the frames are uploaded by knn_rms_run in chunks, overlapped with the
    // superposition of the chunks already on the device
    MDS_TRY(dref.alloc(ctx, sizeof(float) * 3 * (size_t)natoms * n_ref));
    pref = dref.as<float>();
    pl.href = ref_xyz;
    if (fit_xyz) {
      MDS_TRY(dfit.alloc(ctx, sizeof(float) * 3 * (size_t)natoms * n_fit));
      pfit = dfit.as<float>();
      pl.hfit = fit_xyz;
    }
    MDS_TRY(dd.alloc(ctx, sizeof(double) * width * n_fit));
    MDS_TRY(di.alloc(ctx, sizeof(int) * width * n_fit));
    pd = dd.as<double>();
    pi = di.as<int>();
    std::copy(mass, mass + natoms, hmass.begin());
  } else {
    MDS_CUDA(ctx, cudaMemcpyAsync(hmass.data(), mass, sizeof(float) * natoms, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  for (int a = 0; a < natoms; ++a)
    if (!(hmass[a] >= 0.f) || !std::isfinite(hmass[a]))
      return mds_fail(ctx, MDS_ERR_ARG, "mass[%d] is negative or not finite", a);
  MDS_TRY(knn_rms_run(ctx, pl, pref, fit_xyz ? pfit : nullptr, hmass.data(), pd, pi));
  if (!dev && !hooks.screen_keys && !hooks.prep_dev) {
    MDS_CUDA(ctx, cudaMemcpyAsync(out_d, pd, sizeof(double) * width * n_fit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(out_i, pi, sizeof(int) * width * n_fit, cudaMemcpyDeviceToHost, s));
  }
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->stats.total_ms = timer.ms();
  return MDS_OK;
}

int knn_data_run(mds_ctx* ctx, const double* dref, int nref, const double* dfit, int nfit, int dim, int k,
                 bool corr, bool full, unsigned prec, bool noskip, double* dout_d, int* dout_i);

extern "C" int mds_knn_data(mds_ctx* ctx, const double* ref, int n_ref, const double* fit, int n_fit, int dim,
                            int k, unsigned flags, double* out_d, int32_t* out_i, int* k_used) {
  if (!ctx) return MDS_ERR_ARG;
  HostTimer timer;
  ctx->stats = mds_knn_stats{};
  if (!ref || !out_d || !out_i) return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  if (n_ref < 1 || dim < 1 || n_fit < 0)
    return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes: n_ref=%d n_fit=%d dim=%d", n_ref, n_fit, dim);
  if (dim > 8192) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "dim=%d exceeds the supported maximum of 8192", dim);
  const bool full = (flags & MDS_FULL) != 0, dev = (flags & MDS_DEVICE_IO) != 0;
  const bool corr = (flags & MDS_CORRELATION) != 0;
  const unsigned prec = flags & MDS_PREC_MASK;
  if (prec != MDS_PREC_FP32 && prec != MDS_PREC_BF16X3)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "knn_data screen precision 0x%x", prec);
  if (!fit) n_fit = n_ref;
  // knn_data.cpp:186-188: k clamped to N_ref - 1, k1 recomputed
  if (!full) {
    if (k < 0) return mds_fail(ctx, MDS_ERR_ARG, "k must be >= 0");
    if (n_ref - 1 < k) k = n_ref - 1;
    if (k + 1 > 416) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d exceeds the supported maximum of 415", k);
  }
  if (k_used) *k_used = k;
  ctx->stats.pairs = (long long)n_ref * n_fit;
  if (n_fit == 0 || (!full && k == 0)) return MDS_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const size_t width = full ? (size_t)n_ref : (size_t)k;
  DevBuf dref(ctx), dfit(ctx), dd(ctx), di(ctx);
  const double* pr = ref;
  const double* pf = fit;
  double* pd = out_d;
  int* pi = out_i;
  if (!dev) {
    MDS_TRY(dref.alloc(ctx, sizeof(double) * (size_t)dim * n_ref));
    MDS_CUDA(ctx, cudaMemcpyAsync(dref.p, ref, sizeof(double) * (size_t)dim * n_ref, cudaMemcpyHostToDevice, s));
    pr = dref.as<double>();
    if (fit) {
      MDS_TRY(dfit.alloc(ctx, sizeof(double) * (size_t)dim * n_fit));
      MDS_CUDA(ctx, cudaMemcpyAsync(dfit.p, fit, sizeof(double) * (size_t)dim * n_fit, cudaMemcpyHostToDevice, s));
      pf = dfit.as<double>();
    }
    MDS_TRY(dd.alloc(ctx, sizeof(double) * width * n_fit));
    MDS_TRY(di.alloc(ctx, sizeof(int) * width * n_fit));
    pd = dd.as<double>();
    pi = di.as<int>();
  }
  MDS_TRY(knn_data_run(ctx, pr, n_ref, fit ? pf : nullptr, n_fit, dim, k, corr, full, prec,
                       (flags & MDS_NO_SKIP) != 0, pd, pi));
  if (!dev) {
    MDS_CUDA(ctx, cudaMemcpyAsync(out_d, pd, sizeof(double) * width * n_fit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(out_i, pi, sizeof(int) * width * n_fit, cudaMemcpyDeviceToHost, s));
  }
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->stats.total_ms = timer.ms();
  return MDS_OK;
}
