// sparse.cu -- sparse assembly of the neighbour graph on sm_103a:
// make_sysparse (symmetric, one strict triangle) and make_gesparse (general).
//
// Replaces the Berkeley-DB B-tree of make_sysparse.cpp:184-313 /
// make_gesparse.cpp:184-335 (keys ordered by compare_edge, mdsctk.cpp:567-577;
// a put overwrites; the cursor walk of split_edges, mdsctk.cpp:580-604) with
// a sort: every kept (row, neighbour) entry becomes a 64-bit key (from, to)
// in the B-tree's order plus its sequence number in the reference's insertion
// order. A stable LSD radix sort over the key digits that vary, then "last of
// each run of equal keys" is exactly "the last put wins". The cursor walk
// emits column c = the keys whose from == c, in ascending to; it never moves
// past a key whose from is not the current column, so the columns are the
// keys with 0 <= from < n unless the smallest key has from < 0 (then every
// column is empty).
#include <algorithm>
#include <vector>

#include "mds_common.cuh"

#define RS_THREADS 256
#define RS_ITEMS 16
#define RS_TILE (RS_THREADS * RS_ITEMS)

// signed 32-bit -> order-preserving unsigned
__device__ __forceinline__ uint32_t ord32(int v) { return (uint32_t)v ^ 0x80000000u; }
__device__ __forceinline__ int unord32(uint32_t u) { return (int)(u ^ 0x80000000u); }

__global__ void k_scan_int(const int* __restrict__ in, int64_t n, int64_t* __restrict__ out, int64_t* total);

// ---------------------------------------------------------------------------
// key generation, in the reference's insertion order
// ---------------------------------------------------------------------------
// sysparse: for r, x < k: j = idx[r*maxk+x]; r<j -> (r,j); j<r -> (j,r).
// gesparse: (r, j) always; with `sym` (mode 2), also (j, r), inserted only
// where that key is absent when it is put (make_gesparse.cpp:259-271).
// Slot e*2 holds the direct put of entry e = r*k + x, slot e*2+1 the
// transposed one; seq = slot, so seq order is the order of the puts.
__global__ void k_edge_flags(const int* __restrict__ idx, int n, int maxk, int k, int mode, int* __restrict__ flag) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * k) return;
  int r = (int)(e / k), x = (int)(e % k);
  int j = idx[(int64_t)r * maxk + x];
  flag[2 * e] = (mode != 0 || j != r) ? 1 : 0;
  flag[2 * e + 1] = (mode == 2) ? 1 : 0;
}

__global__ void k_edge_write(const int* __restrict__ idx, int n, int maxk, int k, int mode,
                             const int* __restrict__ flag, const int64_t* __restrict__ pos,
                             unsigned long long* __restrict__ keys, int64_t* __restrict__ seq) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * k) return;
  int r = (int)(e / k), x = (int)(e % k);
  int j = idx[(int64_t)r * maxk + x];
  if (flag[2 * e]) {
    int from = r, to = j;
    if (mode == 0 && j < r) { from = j; to = r; }
    keys[pos[2 * e]] = ((unsigned long long)ord32(from) << 32) | ord32(to);
    seq[pos[2 * e]] = 2 * e;
  }
  if (flag[2 * e + 1]) {
    keys[pos[2 * e + 1]] = ((unsigned long long)ord32(j) << 32) | ord32(r);
    seq[pos[2 * e + 1]] = 2 * e + 1;
  }
}

// ---------------------------------------------------------------------------
// LSD radix sort (8-bit digits) of (uint64 key, int64 value), stable
// ---------------------------------------------------------------------------
__global__ void k_rs_hist(const unsigned long long* __restrict__ keys, int64_t n, int shift,
                          unsigned* __restrict__ hist, int nblocks) {
  __shared__ unsigned h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int i = 0; i < RS_ITEMS; ++i) {
    int64_t e = base + (int64_t)i * RS_THREADS + threadIdx.x;
    if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * nblocks + blockIdx.x] = h[d];
}

// exclusive scan of hist (256 * nblocks entries), one block of 1024 threads
__global__ void k_rs_scan(unsigned* __restrict__ hist, int64_t total) {
  __shared__ unsigned long long part[1024];
  int64_t per = (total + blockDim.x - 1) / blockDim.x;
  int64_t b = threadIdx.x * per, e = min(total, b + per);
  unsigned long long s = 0;
  for (int64_t i = b; i < e; ++i) s += hist[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      unsigned long long v = part[i];
      part[i] = acc;
      acc += v;
    }
  }
  __syncthreads();
  unsigned long long acc = part[threadIdx.x];
  for (int64_t i = b; i < e; ++i) {
    unsigned v = hist[i];
    hist[i] = (unsigned)acc;
    acc += v;
  }
}

__global__ void __launch_bounds__(RS_THREADS)
k_rs_scatter(const unsigned long long* __restrict__ kin, const int64_t* __restrict__ vin, int64_t n, int shift,
             const unsigned* __restrict__ hist, int nblocks, unsigned long long* __restrict__ kout,
             int64_t* __restrict__ vout) {
  __shared__ unsigned wcnt[RS_THREADS / 32][256];
  __shared__ unsigned run[256];
  __shared__ unsigned gbase[256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int d = threadIdx.x; d < 256; d += blockDim.x) {
    run[d] = 0;
    gbase[d] = hist[(int64_t)d * nblocks + blockIdx.x];
  }
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int it = 0; it < RS_ITEMS; ++it) {
    for (int i = threadIdx.x; i < (RS_THREADS / 32) * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    int64_t e = base + (int64_t)it * RS_THREADS + threadIdx.x;
    bool valid = e < n;
    unsigned long long key = valid ? kin[e] : 0ull;
    int d = valid ? (int)((key >> shift) & 255) : 256 + lane;  // invalid: unique sentinel
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned lt = peers & ((1u << lane) - 1u);
    int rank = __popc(lt);
    bool leader = (lt == 0);
    if (valid && leader) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (valid) {
      unsigned off = run[d] + rank;
      for (int w = 0; w < warp; ++w) off += wcnt[w][d];
      int64_t pos = (int64_t)gbase[d] + off;
      kout[pos] = key;
      vout[pos] = vin[e];
    }
    __syncthreads();
    for (int dd = threadIdx.x; dd < 256; dd += blockDim.x) {
      unsigned s = 0;
      for (int w = 0; w < RS_THREADS / 32; ++w) s += wcnt[w][dd];
      run[dd] += s;
    }
    __syncthreads();
  }
}

__global__ void k_or_diff(const unsigned long long* __restrict__ keys, int64_t n,
                          unsigned long long* __restrict__ out) {
  __shared__ unsigned long long s[256];
  unsigned long long k0 = keys[0], acc = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    acc |= keys[e] ^ k0;
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] |= s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicOr(out, s[0]);
}

// Stable sort of n (key, value) pairs by the key bits in `mask`; ping-pongs
// between (k0,v0) and (k1,v1); returns the index (0/1) holding the result.
int radix_sort(mds_ctx* ctx, unsigned long long* k0, int64_t* v0, unsigned long long* k1, int64_t* v1,
               int64_t n, unsigned long long mask, int* which) {
  cudaStream_t s = ctx->stream;
  *which = 0;
  if (n <= 1) return MDS_OK;
  const int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
  DevBuf hist(ctx);
  MDS_TRY(hist.alloc(ctx, sizeof(unsigned) * 256 * (size_t)nblocks));
  unsigned long long* ka = k0;
  int64_t* va = v0;
  unsigned long long* kb = k1;
  int64_t* vb = v1;
  for (int shift = 0; shift < 64; shift += 8) {
    if (((mask >> shift) & 255ull) == 0) continue;
    ctx->stats.launches += 3;
    k_rs_hist<<<nblocks, RS_THREADS, 0, s>>>(ka, n, shift, hist.as<unsigned>(), nblocks);
    k_rs_scan<<<1, 1024, 0, s>>>(hist.as<unsigned>(), (int64_t)256 * nblocks);
    k_rs_scatter<<<nblocks, RS_THREADS, 0, s>>>(ka, va, n, shift, hist.as<unsigned>(), nblocks, kb, vb);
    MDS_CUDA(ctx, cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
    *which ^= 1;
  }
  return MDS_OK;
}

// ---------------------------------------------------------------------------
// resolution of the puts and CSC emission
// ---------------------------------------------------------------------------
// Keys sorted by (key, seq). Symmetric / plain general mode: keep the last
// entry of each run of equal keys (last put wins). General with `sym`:
// a transposed put (odd seq) only inserts when the key is absent, so in a
// run the winner is the last direct put if any, else the first transposed
// put; later transposed puts never overwrite.
__global__ void k_resolve(const unsigned long long* __restrict__ keys, const int64_t* __restrict__ seq, int64_t n,
                          int mode, int* __restrict__ keep) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  bool last = (e + 1 == n) || keys[e + 1] != keys[e];
  if (mode != 2) {
    keep[e] = last ? 1 : 0;
    return;
  }
  // run boundaries
  bool first = (e == 0) || keys[e - 1] != keys[e];
  bool direct = (seq[e] & 1) == 0;
  int k = 0;
  if (direct) {
    // winner if no later direct put of the same key: the direct puts are the
    // even seq values; a later transposed put can only overwrite ... never.
    // Is there a later direct put in this run?
    int64_t f = e + 1;
    bool later = false;
    while (f < n && keys[f] == keys[e]) {
      if ((seq[f] & 1) == 0) { later = true; break; }
      ++f;
    }
    k = later ? 0 : 1;
    // a direct put that follows a transposed insert overwrites it; the
    // transposed one is then dropped below.
  } else {
    // transposed put: effective only if no direct put of this key came
    // before it (then the key was absent) and it is the first transposed
    // put of the run; it is then replaced by any later direct put.
    bool earlier = false;
    for (int64_t f = e - 1; f >= 0 && keys[f] == keys[e]; --f)
      earlier = true;  // any earlier put (direct or transposed) means present
    bool later_direct = false;
    for (int64_t f = e + 1; f < n && keys[f] == keys[e]; ++f)
      if ((seq[f] & 1) == 0) { later_direct = true; break; }
    k = (!earlier && !later_direct) ? 1 : 0;
    (void)first;
  }
  keep[e] = k;
}

// exclusive scan helper for int arrays (one block, chunked)
__global__ void k_scan_int(const int* __restrict__ in, int64_t n, int64_t* __restrict__ out, int64_t* total) {
  __shared__ long long part[1024];
  int64_t per = (n + blockDim.x - 1) / blockDim.x;
  int64_t b = threadIdx.x * per, e = min(n, b + per);
  long long s = 0;
  for (int64_t i = b; i < e; ++i) s += in[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      long long v = part[i];
      part[i] = acc;
      acc += v;
    }
    *total = acc;
  }
  __syncthreads();
  long long acc = part[threadIdx.x];
  for (int64_t i = b; i < e; ++i) {
    out[i] = acc;
    acc += in[i];
  }
}

// compact kept entries with 0 <= from < ncol into (from, to, val)
__global__ void k_emit(const unsigned long long* __restrict__ keys, const int64_t* __restrict__ seq,
                       const int* __restrict__ keep, const int64_t* __restrict__ pos, int64_t n,
                       const double* __restrict__ dist, int maxk, int k, int ncol, int* __restrict__ colof,
                       int* __restrict__ irow, double* __restrict__ val) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n || !keep[e]) return;
  int from = unord32((uint32_t)(keys[e] >> 32));
  int to = unord32((uint32_t)(keys[e] & 0xffffffffu));
  if (from < 0 || from >= ncol) return;
  int64_t s = seq[e] >> 1;  // r * k + x
  int r = (int)(s / k), x = (int)(s % k);
  int64_t p = pos[e];
  colof[p] = from;
  irow[p] = to;
  val[p] = dist[(int64_t)r * maxk + x];
}

__global__ void k_pcol(const int* __restrict__ colof, int64_t nnz, int ncol, int* __restrict__ pcol) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncol) return;
  // lower_bound of c in colof (ascending)
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (colof[mid] < c) lo = mid + 1; else hi = mid;
  }
  pcol[c] = (int)lo;
}

__global__ void k_keep_inrange(const unsigned long long* __restrict__ keys, int64_t n, int ncol,
                               int* __restrict__ keep) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  int from = unord32((uint32_t)(keys[e] >> 32));
  if (from < 0 || from >= ncol) keep[e] = 0;
}

// mode 0: sysparse; 1: gesparse; 2: gesparse with -s
static int assemble(mds_ctx* ctx, const double* ddist, const int* didx, int n, int maxk, int k, int mode,
                    int* dpcol, int* dirow, double* dval, int64_t cap, int64_t* nnz_out) {
  cudaStream_t s = ctx->stream;
  const int64_t nent = (int64_t)n * k * (mode == 2 ? 2 : 1);  // keys at most
  DevBuf k0(ctx), v0(ctx), k1(ctx), v1(ctx), diff(ctx), keep(ctx), pos(ctx), total(ctx), colof(ctx);
  MDS_TRY(k0.alloc(ctx, sizeof(unsigned long long) * std::max<int64_t>(nent, 1)));
  MDS_TRY(v0.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(nent, 1)));
  MDS_TRY(k1.alloc(ctx, sizeof(unsigned long long) * std::max<int64_t>(nent, 1)));
  MDS_TRY(v1.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(nent, 1)));
  MDS_TRY(diff.alloc(ctx, sizeof(unsigned long long)));
  MDS_CUDA(ctx, cudaMemsetAsync(diff.p, 0, sizeof(unsigned long long), s));
  int64_t m = 0;
  {
    const int64_t slots = (int64_t)n * k * 2;
    DevBuf flag(ctx), fpos(ctx), ftot(ctx);
    MDS_TRY(flag.alloc(ctx, sizeof(int) * std::max<int64_t>(slots, 1)));
    MDS_TRY(fpos.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(slots, 1)));
    MDS_TRY(ftot.alloc(ctx, sizeof(int64_t)));
    MDS_CUDA(ctx, cudaMemsetAsync(ftot.p, 0, sizeof(int64_t), s));
    if (slots > 0) {
      const int g = (int)(((int64_t)n * k + 255) / 256);
      ctx->stats.launches += 3;
      k_edge_flags<<<g, 256, 0, s>>>(didx, n, maxk, k, mode, flag.as<int>());
      k_scan_int<<<1, 1024, 0, s>>>(flag.as<int>(), slots, fpos.as<int64_t>(), ftot.as<int64_t>());
      k_edge_write<<<g, 256, 0, s>>>(didx, n, maxk, k, mode, flag.as<int>(), fpos.as<int64_t>(),
                                     k0.as<unsigned long long>(), v0.as<int64_t>());
      MDS_CUDA(ctx, cudaGetLastError());
    }
    MDS_CUDA(ctx, cudaMemcpyAsync(&m, ftot.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  int which = 0;
  if (m > 1) {
    ctx->stats.launches++;
    k_or_diff<<<(int)std::min<int64_t>((m + 255) / 256, 1024), 256, 0, s>>>(k0.as<unsigned long long>(), m,
                                                                          diff.as<unsigned long long>());
    MDS_CUDA(ctx, cudaGetLastError());
    unsigned long long mask = 0;
    MDS_CUDA(ctx, cudaMemcpyAsync(&mask, diff.p, sizeof(mask), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    MDS_TRY(radix_sort(ctx, k0.as<unsigned long long>(), v0.as<int64_t>(), k1.as<unsigned long long>(),
                       v1.as<int64_t>(), m, mask, &which));
  }
  unsigned long long* keys = which ? k1.as<unsigned long long>() : k0.as<unsigned long long>();
  int64_t* seq = which ? v1.as<int64_t>() : v0.as<int64_t>();
  MDS_TRY(keep.alloc(ctx, sizeof(int) * std::max<int64_t>(m, 1)));
  MDS_TRY(pos.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(m, 1)));
  MDS_TRY(total.alloc(ctx, sizeof(int64_t)));
  // the cursor walk: nothing is emitted if the smallest key's from < 0
  bool blocked = false;
  if (m > 0) {
    unsigned long long first = 0;
    MDS_CUDA(ctx, cudaMemcpyAsync(&first, keys, sizeof(first), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    int from0 = (int)((uint32_t)(first >> 32) ^ 0x80000000u);
    blocked = from0 < 0;
  }
  int64_t nnz = 0;
  if (m > 0 && !blocked) {
    ctx->stats.launches += 3;
    k_resolve<<<(int)((m + 255) / 256), 256, 0, s>>>(keys, seq, m, mode, keep.as<int>());
    k_keep_inrange<<<(int)((m + 255) / 256), 256, 0, s>>>(keys, m, n, keep.as<int>());
    k_scan_int<<<1, 1024, 0, s>>>(keep.as<int>(), m, pos.as<int64_t>(), total.as<int64_t>());
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaMemcpyAsync(&nnz, total.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  if (nnz > cap) return mds_fail(ctx, MDS_ERR_ARG, "output capacity %lld < nnz %lld", (long long)cap, (long long)nnz);
  MDS_TRY(colof.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz, 1)));
  if (nnz > 0) {
    ctx->stats.launches++;
    k_emit<<<(int)((m + 255) / 256), 256, 0, s>>>(keys, seq, keep.as<int>(), pos.as<int64_t>(), m, ddist, maxk, k, n,
                                                colof.as<int>(), dirow, dval);
  }
  ctx->stats.launches++;
  k_pcol<<<(n + 1 + 255) / 256, 256, 0, s>>>(colof.as<int>(), nnz, n, dpcol);
  MDS_CUDA(ctx, cudaGetLastError());
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  *nnz_out = nnz;
  return MDS_OK;
}

static int assemble_api(mds_ctx* ctx, const double* dist, const int32_t* idx, int n_rows, int maxk, int k,
                        unsigned flags, int mode, int32_t* pcol, int32_t* irow, double* val, int64_t cap,
                        int64_t* nnz) {
  if (!ctx) return MDS_ERR_ARG;
  ctx->stats = mds_knn_stats{};
  if (!dist || !idx || !pcol || !irow || !val || !nnz) return mds_fail(ctx, MDS_ERR_ARG, "null argument");
  if (n_rows < 0 || maxk < 1 || k < 0 || k > maxk)
    return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes n_rows=%d maxk=%d k=%d (need k <= maxk)", n_rows, maxk, k);
  if ((int64_t)n_rows * k * 2 >= (1ll << 40)) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "too many entries");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const bool dev = (flags & MDS_DEVICE_IO) != 0;
  DevBuf dd(ctx), di(ctx), dp(ctx), dr(ctx), dv(ctx);
  const double* pdist = dist;
  const int* pidx = idx;
  int* ppcol = pcol;
  int* pirow = irow;
  double* pval = val;
  const size_t ent = (size_t)n_rows * maxk;
  if (!dev) {
    MDS_TRY(dd.alloc(ctx, sizeof(double) * std::max<size_t>(ent, 1)));
    MDS_TRY(di.alloc(ctx, sizeof(int) * std::max<size_t>(ent, 1)));
    if (ent) {
      MDS_CUDA(ctx, cudaMemcpyAsync(dd.p, dist, sizeof(double) * ent, cudaMemcpyHostToDevice, s));
      MDS_CUDA(ctx, cudaMemcpyAsync(di.p, idx, sizeof(int) * ent, cudaMemcpyHostToDevice, s));
    }
    MDS_TRY(dp.alloc(ctx, sizeof(int) * (n_rows + 1)));
    MDS_TRY(dr.alloc(ctx, sizeof(int) * std::max<int64_t>(cap, 1)));
    MDS_TRY(dv.alloc(ctx, sizeof(double) * std::max<int64_t>(cap, 1)));
    pdist = dd.as<double>();
    pidx = di.as<int>();
    ppcol = dp.as<int>();
    pirow = dr.as<int>();
    pval = dv.as<double>();
  }
  int64_t m = 0;
  MDS_TRY(assemble(ctx, pdist, pidx, n_rows, maxk, k, mode, ppcol, pirow, pval, cap, &m));
  if (!dev) {
    MDS_CUDA(ctx, cudaMemcpyAsync(pcol, ppcol, sizeof(int) * (n_rows + 1), cudaMemcpyDeviceToHost, s));
    if (m) {
      MDS_CUDA(ctx, cudaMemcpyAsync(irow, pirow, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaMemcpyAsync(val, pval, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    }
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  *nnz = m;
  return MDS_OK;
}

extern "C" int mds_sysparse(mds_ctx* ctx, const double* dist, const int32_t* idx, int n_rows, int maxk, int k,
                            unsigned flags, int32_t* pcol, int32_t* irow, double* val, int64_t cap,
                            int64_t* nnz) {
  return assemble_api(ctx, dist, idx, n_rows, maxk, k, flags, 0, pcol, irow, val, cap, nnz);
}

extern "C" int mds_gesparse(mds_ctx* ctx, const double* dist, const int32_t* idx, int n_rows, int maxk, int k,
                            int symmetric, unsigned flags, int32_t* pcol, int32_t* irow, double* val,
                            int64_t cap, int64_t* nnz) {
  return assemble_api(ctx, dist, idx, n_rows, maxk, k, flags, symmetric ? 2 : 1, pcol, irow, val, cap, nnz);
}
