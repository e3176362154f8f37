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

extern "C" int mds_knn_rms(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz,
                           int n_fit, int natoms, const float* mass, int k, unsigned flags,
                           double* out_d, int32_t* out_i, int* k_used) {
  if (!ctx) return MDS_ERR_ARG;
  HostTimer timer;
  ctx->stats = mds_knn_stats{};
  if (!ref_xyz || !mass || !out_d || !out_i)
    return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
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
  pl.prec = prec;
  pl.kprime = std::min(mds_round_up(std::max(k + 1 + 32, (k + 1) * 3 / 2), 32), 448);
  pl.guard_fp32 = 1.0f / 65536.0f;
  pl.guard_tc = 1.0f / 8192.0f;
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
    MDS_TRY(dref.alloc(ctx, sizeof(float) * 3 * (size_t)natoms * n_ref));
    MDS_CUDA(ctx, cudaMemcpyAsync(dref.p, ref_xyz, sizeof(float) * 3 * (size_t)natoms * n_ref,
                                  cudaMemcpyHostToDevice, s));
    pref = dref.as<float>();
    if (fit_xyz) {
      MDS_TRY(dfit.alloc(ctx, sizeof(float) * 3 * (size_t)natoms * n_fit));
      MDS_CUDA(ctx, cudaMemcpyAsync(dfit.p, fit_xyz, sizeof(float) * 3 * (size_t)natoms * n_fit,
                                    cudaMemcpyHostToDevice, s));
      pfit = dfit.as<float>();
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
  if (!dev) {
    MDS_CUDA(ctx, cudaMemcpyAsync(out_d, pd, sizeof(double) * width * n_fit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(out_i, pi, sizeof(int) * width * n_fit, cudaMemcpyDeviceToHost, s));
  }
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->stats.total_ms = timer.ms();
  return MDS_OK;
}

extern "C" int mds_knn_data(mds_ctx* ctx, const double*, int, const double*, int, int, int, unsigned,
                            double*, int32_t*, int*) {
  return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "knn_data not built yet");
}
