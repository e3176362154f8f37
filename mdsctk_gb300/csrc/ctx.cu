// ctx.cu -- context lifecycle, error reporting and version of libmdsgpu.
#include "mds_common.cuh"

int mds_fail(mds_ctx* ctx, int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->last_error = buf;
  return code;
}

void mds_trim_cache(mds_ctx* ctx, size_t keep) {
  if (!ctx || ctx->cache.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  size_t cached = 0;
  for (auto& kv : ctx->cache) cached += kv.first;
  while (!ctx->cache.empty() && cached > keep) {
    auto it = std::prev(ctx->cache.end());  // largest first
    cudaFree(it->second);
    cached -= it->first;
    ctx->hbm_in_use -= it->first;
    ctx->cache.erase(it);
  }
}

int mds_upload_chunked(mds_ctx* ctx, void* dst, const void* src, int n, size_t frame_bytes, int ev0,
                       std::vector<int>& bounds, int* nchunks, int align) {
  if (!ctx->order_ev) {
    for (auto& cs : ctx->copy_stream) MDS_CUDA(ctx, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    for (auto& e : ctx->chunk_ev) MDS_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    MDS_CUDA(ctx, cudaEventCreateWithFlags(&ctx->order_ev, cudaEventDisableTiming));
  }
  // chunks of at least 4 MiB, at most MDS_MAX_CHUNKS
  const size_t total = frame_bytes * (size_t)n;
  int c = (int)std::min<size_t>(MDS_MAX_CHUNKS, std::max<size_t>(1, total >> 22));
  align = std::max(align, 1);
  c = std::max(1, std::min(c, n / align));
  bounds.resize(c + 1);
  for (int i = 0; i <= c; ++i) bounds[i] = (i == c) ? n : (int)((int64_t)n * i / c / align * align);
  // (bounds stay strictly increasing: consecutive ones are at least
  // n / c >= align frames apart before rounding down to the alignment)
  // the destination may be a cached block last used by work on ctx->stream
  MDS_CUDA(ctx, cudaEventRecord(ctx->order_ev, ctx->stream));
  for (auto cs : ctx->copy_stream) MDS_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->order_ev, 0));
  // All chunks on one copy stream, so they land in order. The host link
  // carries ~205 GB/s whichever way the copies are issued (one or several
  // streams, or a kernel reading the mapped host memory); with the chunks
  // alternating between two streams, one copy engine served every chunk of
  // one stream before any of the other's, and the first chunk landed last
  // but one.
  cudaStream_t cs = ctx->copy_stream[0];
  for (int i = 0; i < c; ++i) {
    const size_t off = frame_bytes * (size_t)bounds[i], bytes = frame_bytes * (size_t)(bounds[i + 1] - bounds[i]);
    MDS_CUDA(ctx, cudaMemcpyAsync(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, bytes,
                                  cudaMemcpyHostToDevice, cs));
    MDS_CUDA(ctx, cudaEventRecord(ctx->chunk_ev[ev0 + i], cs));
  }
  *nchunks = c;
  return MDS_OK;
}

extern "C" const char* mds_version(void) { return "mdsgpu 0.1 (sm_103a)"; }

extern "C" int mds_create(int device, size_t hbm_budget, mds_ctx** out) {
  if (!out) return MDS_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MDS_ERR_CUDA;
  if (device < 0 || device >= ndev) return MDS_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MDS_ERR_CUDA;
  mds_ctx* c = new mds_ctx();
  c->device = device;
  c->hbm_budget = hbm_budget;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return MDS_ERR_CUDA;
  }
  for (auto& e : c->ev) cudaEventCreate(&e);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return MDS_OK;
}

extern "C" int mds_destroy(mds_ctx* ctx) {
  if (!ctx) return MDS_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  mds_trim_cache(ctx, 0);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : ctx->chunk_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->order_ev) cudaEventDestroy(ctx->order_ev);
  for (auto cs : ctx->copy_stream)
    if (cs) {
      cudaStreamSynchronize(cs);
      cudaStreamDestroy(cs);
    }
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MDS_OK;
}

extern "C" const char* mds_last_error(const mds_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int mds_get_knn_stats(const mds_ctx* ctx, mds_knn_stats* out) {
  if (!ctx || !out) return MDS_ERR_ARG;
  *out = ctx->stats;
  return MDS_OK;
}

extern "C" int mds_test_inject(mds_ctx* ctx, unsigned what) {
  if (!ctx) return MDS_ERR_ARG;
  if (what & ~MDS_INJECT_SCREEN_STALL) return mds_fail(ctx, MDS_ERR_ARG, "unknown fault 0x%x", what);
  ctx->inject = what;
  return MDS_OK;
}
