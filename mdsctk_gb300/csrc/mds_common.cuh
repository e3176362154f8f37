// mds_common.cuh -- shared definitions of libmdsgpu (context, errors,
// device workspace, small device helpers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "../../include/mdsgpu.h"

#define MDS_MAX_CHUNKS 8  // chunks of a pipelined frame upload

struct mds_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t hbm_budget = 0;  // 0 = no limit beyond what cudaMalloc gives
  size_t hbm_in_use = 0;  // bytes held by live buffers and by the cache
  // Freed device blocks kept for reuse by later calls (size -> pointer).
  // Every use of a block is ordered on `stream`, so a block returned here can
  // be handed out again without synchronising.
  std::multimap<size_t, void*> cache;
  std::string last_error;
  int num_sms = 0;
  // statistics of the last kNN call (exposed through mds_knn_stats)
  mds_knn_stats stats{};
  // timing of the last call's dominant kernel (CUDA events on ctx->stream)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // host-to-device uploads in chunks (created on first use): a copy
  // stream, one event per chunk, one event ordering the copies after the
  // work already queued on `stream`
  cudaStream_t copy_stream[1] = {nullptr};
  cudaEvent_t chunk_ev[MDS_MAX_CHUNKS * 2] = {};
  cudaEvent_t order_ev = nullptr;
  // mds_test_inject: faults armed for the next call that reaches them
  unsigned inject = 0;
};

// Record an error message on the context and return `code`.
int mds_fail(mds_ctx* ctx, int code, const char* fmt, ...);

// Upload n frames of `frame_bytes` each from host memory to dst in up to
// MDS_MAX_CHUNKS chunks, in order on the context's first copy stream and
// ordered after the work already queued on ctx->stream. Chunk c covers
// frames [bounds[c], bounds[c+1]) and completes event ctx->chunk_ev[ev0 + c];
// the consumer waits on that event before reading the chunk. From pageable
// host memory the copies are correct but do not overlap. Returns the number
// of chunks through *nchunks. Inner chunk bounds are multiples of `align`
// frames.
int mds_upload_chunked(mds_ctx* ctx, void* dst, const void* src, int n, size_t frame_bytes, int ev0,
                       std::vector<int>& bounds, int* nchunks, int align = 1);

// Free cached device blocks until at most `keep` bytes remain cached
// (synchronises the context's stream first).
void mds_trim_cache(mds_ctx* ctx, size_t keep);

#define MDS_CUDA(ctx, call)                                                        \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess)                                                         \
      return mds_fail((ctx), MDS_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, \
                      cudaGetErrorString(_e));                                     \
  } while (0)

// Device buffer owned by a context; freed on scope exit. Accounts against the
// context's HBM budget.
struct DevBuf {
  mds_ctx* ctx = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  explicit DevBuf(mds_ctx* c) : ctx(c) {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && ctx) ctx->cache.emplace(bytes, p);  // stays counted in hbm_in_use
    p = nullptr;
    bytes = 0;
  }
  // Returns MDS_OK or an error code (recorded on ctx). Sizes are rounded up
  // to 4 KiB; a cached block of up to twice the size is reused.
  int alloc(mds_ctx* c, size_t n) {
    release();
    ctx = c;
    n = (std::max<size_t>(n, 16) + 4095) & ~(size_t)4095;
    auto it = ctx->cache.lower_bound(n);
    if (it != ctx->cache.end() && it->first <= 2 * n) {
      bytes = it->first;
      p = it->second;
      ctx->cache.erase(it);
      return MDS_OK;
    }
    if (ctx->hbm_budget && ctx->hbm_in_use + n > ctx->hbm_budget) mds_trim_cache(ctx, 0);
    if (ctx->hbm_budget && ctx->hbm_in_use + n > ctx->hbm_budget)
      return mds_fail(ctx, MDS_ERR_NOMEM, "HBM budget exceeded: need %zu more bytes (in use %zu, budget %zu)",
                      n, ctx->hbm_in_use, ctx->hbm_budget);
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      mds_trim_cache(ctx, 0);
      e = cudaMalloc(&p, n);
    }
    if (e != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return mds_fail(ctx, MDS_ERR_NOMEM, "cudaMalloc(%zu): %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    ctx->hbm_in_use += n;
    return MDS_OK;
  }
  template <class T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

#define MDS_TRY(expr)              \
  do {                             \
    int _r = (expr);               \
    if (_r != MDS_OK) return _r;   \
  } while (0)

// Let `kernel` use all the dynamic shared memory the device allows next to its
// static shared memory. Done once per kernel (*done), so that later launches
// (also those made while a stream is captured) need no attribute call.
template <class Kernel>
int mds_allow_dyn_smem(mds_ctx* ctx, Kernel kernel, bool* done, size_t* limit) {
  if (!*done) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return mds_fail(ctx, MDS_ERR_CUDA, "cudaFuncGetAttributes");
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    int dyn = optin - (int)fa.sharedSizeBytes;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    if (e != cudaSuccess)
      return mds_fail(ctx, MDS_ERR_CUDA, "cudaFuncSetAttribute(%d): %s", dyn, cudaGetErrorString(e));
    *limit = (size_t)dyn;
    *done = true;
  }
  return MDS_OK;
}

static inline int mds_round_up(int x, int m) { return (x + m - 1) / m * m; }

// Stable LSD radix sort (8-bit digits over the bits set in `mask`) of n
// (uint64 key, int64 value) pairs, ping-ponging between (k0,v0) and (k1,v1);
// *which = 1 if the result ended in (k1,v1) (sparse.cu).
int radix_sort(mds_ctx* ctx, unsigned long long* k0, int64_t* v0, unsigned long long* k1, int64_t* v1,
               int64_t n, unsigned long long mask, int* which);

// Pack a non-negative float key and an index into one ordered 64-bit word:
// ascending order = ascending (value, index).
__host__ __device__ __forceinline__ uint64_t mds_pack_key(float s, int j) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(s);
#else
  uint32_t u;
  std::memcpy(&u, &s, 4);
#endif
  return ((uint64_t)u << 32) | (uint32_t)j;
}
__host__ __device__ __forceinline__ float mds_key_value(uint64_t k) {
#ifdef __CUDA_ARCH__
  return __uint_as_float((uint32_t)(k >> 32));
#else
  uint32_t u = (uint32_t)(k >> 32);
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ int mds_key_index(uint64_t k) { return (int)(uint32_t)(k & 0xffffffffu); }

#define MDS_KEY_INF 0xffffffffffffffffull
