// knn_sparse.cu -- knn_data_sparse and contact_profile on sm_103a.
//
// knn_data_sparse (knn_data_sparse.cpp:141-260): k nearest sparse vectors by
// euclidean_distance_sparse (mdsctk.cpp:362-386). Every distance is the
// reference's merge walk restated operation for operation: over the
// reference vector's entries, the fit-only entries with smaller index first
// (their squares), then the matched difference or the reference entry
// squared, each product and sum an FP64 operation in the reference's order,
// so the written distances are bit-identical. One block per fit vector keeps
// it in shared memory; each thread walks one reference vector at a time;
// the k+1 best (value, index) pairs are kept by a bitonic merge per chunk of
// 1,024 reference vectors; position 0 is dropped as in the reference.
//
// contact_profile (contact_profile.cpp:200-262): for every frame the grid
// of atom pairs (g1[i], g2[j]) is tested for distance < eps Angstrom,
// written as the ascending grid indices i * n2 + j of the contacts. The
// reference forms the distance from float differences and float squares
// summed into a double, sqrt, times 10; a pair is decided in FP32 when its
// distance is more than 1e-5 (relative) from eps, and otherwise in the
// reference's arithmetic, so the contact sets are identical.
#include <algorithm>
#include <cmath>
#include <vector>

#include "knn_common.cuh"

#define SP_THREADS 256
#define SP_CHUNK 1024
#define SP_FIT_CAP 2048  // fit entries kept in shared memory (beyond: read from global)

// euclidean_distance_sparse(ref, fit) squared, in the reference's operation
// order (the walk does not assume sorted indices: it is the same walk).
__device__ __forceinline__ double sparse_dist2(const int* __restrict__ ri, const double* __restrict__ rd, int ref_size,
                                               const int* fi, const double* fd, int fit_size) {
  double value = 0.0;
  int f = 0;
  for (int r = 0; r < ref_size; ++r) {
    const int rix = __ldg(ri + r);
    const double rv = __ldg(rd + r);
    while (f < fit_size && fi[f] < rix) {
      value = __dadd_rn(value, __dmul_rn(fd[f], fd[f]));
      ++f;
    }
    if (f < fit_size && rix == fi[f]) {
      const double t = __dsub_rn(rv, fd[f]);
      value = __dadd_rn(value, __dmul_rn(t, t));
      ++f;
    } else {
      value = __dadd_rn(value, __dmul_rn(rv, rv));
    }
  }
  for (; f < fit_size; ++f) value = __dadd_rn(value, __dmul_rn(fd[f], fd[f]));
  return value;
}

// One block per fit vector. mode 0: the k+1 best, position 0 dropped, k per
// row; mode 1 (the reference's -s false): the full row of distances in
// reference order.
__global__ void __launch_bounds__(SP_THREADS)
k_sparse_knn(const int64_t* __restrict__ ref_off, const int* __restrict__ ref_idx, const double* __restrict__ ref_val,
             int nref, const int64_t* __restrict__ fit_off, const int* __restrict__ fit_idx,
             const double* __restrict__ fit_val, int k, int mode, double* __restrict__ out_d,
             int* __restrict__ out_i) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int row = blockIdx.x;
  const int64_t f0 = fit_off[row];
  const int fit_size = (int)(fit_off[row + 1] - f0);
  const int k1 = k + 1;
  const int BP2 = next_pow2(k1 + SP_CHUNK);
  double* bval = reinterpret_cast<double*>(smem_raw);                   // [BP2] (mode 0)
  int* bidx = reinterpret_cast<int*>(bval + (mode == 0 ? BP2 : 0));     // [BP2]
  double* sfd = reinterpret_cast<double*>(bidx + (mode == 0 ? BP2 : 0));  // [SP_FIT_CAP]
  int* sfi = reinterpret_cast<int*>(sfd + SP_FIT_CAP);                  // [SP_FIT_CAP]
  const bool in_smem = fit_size <= SP_FIT_CAP;
  if (in_smem)
    for (int e = threadIdx.x; e < fit_size; e += blockDim.x) {
      sfi[e] = fit_idx[f0 + e];
      sfd[e] = fit_val[f0 + e];
    }
  const int* fi = in_smem ? sfi : fit_idx + f0;
  const double* fd = in_smem ? sfd : fit_val + f0;
  __syncthreads();
  auto dist2 = [&](int j) {
    const int64_t r0 = ref_off[j];
    return sparse_dist2(ref_idx + r0, ref_val + r0, (int)(ref_off[j + 1] - r0), fi, fd, fit_size);
  };
  if (mode == 1) {
    for (int j = threadIdx.x; j < nref; j += blockDim.x) {
      out_d[(int64_t)row * nref + j] = sqrt(dist2(j));
      out_i[(int64_t)row * nref + j] = j;
    }
    return;
  }
  const double INF = __longlong_as_double(0x7ff0000000000000ll);
  for (int x = threadIdx.x; x < BP2; x += blockDim.x) {
    bval[x] = INF;
    bidx[x] = 0x7fffffff;
  }
  __syncthreads();
  for (int base = 0; base < nref; base += SP_CHUNK) {
    const int nc = min(SP_CHUNK, nref - base);
    for (int c = threadIdx.x; c < BP2 - k1; c += blockDim.x) {
      bval[k1 + c] = (c < nc) ? dist2(base + c) : INF;
      bidx[k1 + c] = (c < nc) ? base + c : 0x7fffffff;
    }
    __syncthreads();
    // bitonic sort of (value, index) pairs; the first k1 are the best so far
    for (int kk = 2; kk <= BP2; kk <<= 1)
      for (int jj = kk >> 1; jj > 0; jj >>= 1) {
        for (int i = threadIdx.x; i < BP2; i += blockDim.x) {
          const int ixj = i ^ jj;
          if (ixj > i) {
            const double va = bval[i], vb = bval[ixj];
            const int ia = bidx[i], ib = bidx[ixj];
            // non-negative values: bit patterns order as unsigned integers
            const unsigned long long ua = __double_as_longlong(va), ub = __double_as_longlong(vb);
            const bool gt = (ua > ub) || (ua == ub && ia > ib);
            if (gt == ((i & kk) == 0)) {
              bval[i] = vb; bval[ixj] = va;
              bidx[i] = ib; bidx[ixj] = ia;
            }
          }
        }
        __syncthreads();
      }
  }
  for (int x = threadIdx.x; x < k; x += blockDim.x) {
    out_d[(int64_t)row * k + x] = sqrt(bval[x + 1]);
    out_i[(int64_t)row * k + x] = bidx[x + 1];
  }
}

static size_t sparse_knn_smem(int k, int mode) {
  const size_t fit = (size_t)SP_FIT_CAP * (8 + 4);
  if (mode == 1) return fit;
  return (size_t)next_pow2(k + 1 + SP_CHUNK) * (8 + 4) + fit;
}

// ---------------------------------------------------------------------------
// knn_data_sparse on binary vectors (every value 1.0, indices strictly
// ascending: what contact_profile writes). The reference's walk then adds
// 1.0 for every index in one vector only and 0.0 for every shared index, so
// its FP64 sum is the integer |A| + |B| - 2 |A & B| whatever the order, and
// sqrt of it is the reference's distance bit for bit. The vectors become
// bit sets and |A & B| a popcount tile product: 32 fit rows x 64 reference
// rows per block tile, 2 x 4 pairs per thread, bit-set words staged through
// shared memory by cp.async; the squared distances are exact integers, so
// each row's k+1 smallest (value, index) keys are kept directly (reference
// tiles are visited in index order, so a later tie never displaces an earlier
// one) and no recheck is needed.
// ---------------------------------------------------------------------------
#define BN_TM 32
#define BN_TN 64
#define BN_KW 32  // words per K-chunk
#define BN_WS 36  // words per staged row (bank spread, 16-byte rows)

// CSR rows -> bit sets [n][W] (W words of 32 bits, zero padded)
__global__ void k_bitset(const int64_t* __restrict__ off, const int* __restrict__ idx, int W,
                         unsigned* __restrict__ bits) {
  const int r = blockIdx.x;
  unsigned* b = bits + (int64_t)r * W;
  for (int64_t e = off[r] + threadIdx.x; e < off[r + 1]; e += blockDim.x) {
    const int i = idx[e];
    atomicOr(b + (i >> 5), 1u << (i & 31));
  }
}

__device__ __forceinline__ void cpa16b(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0));
}

__global__ void __launch_bounds__(SP_THREADS)
k_bin_knn(const unsigned* __restrict__ Bf, const int* __restrict__ cf, int nfit, const unsigned* __restrict__ Br,
          const int* __restrict__ cr, int nref, int W, int k, double* __restrict__ out_d, int* __restrict__ out_i) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned* sf = reinterpret_cast<unsigned*>(smem_raw);  // [2][BN_TM * BN_WS]
  unsigned* sr = sf + 2 * BN_TM * BN_WS;                   // [2][BN_TN * BN_WS]
  int* scr = reinterpret_cast<int*>(sr + 2 * BN_TN * BN_WS);  // [BN_TN] column counts
  int* scnt = scr + BN_TN;                                   // [BN_TM]
  float* sthr = reinterpret_cast<float*>(scnt + BN_TM);      // [BN_TM]
  uint64_t* pool = reinterpret_cast<uint64_t*>(sthr + BN_TM);
  const int k1 = k + 1;
  const int P2 = next_pow2(k1 + BN_TN);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, lane = tid & 31, warp = tid >> 5;
  const int row0 = blockIdx.x * BN_TM;
  int cnt_f[2];
  for (int p = 0; p < 2; ++p) {
    const int r = row0 + ty + 16 * p;
    cnt_f[p] = (r < nfit) ? cf[r] : 0;
  }
  if (tid < BN_TM) {
    scnt[tid] = 0;
    sthr[tid] = __int_as_float(0x7f800000);
  }
  const int nch = W / BN_KW;
  const int ntiles = (nref + BN_TN - 1) / BN_TN;
  auto load = [&](int stage, int tile, int kc) {
    unsigned* df = sf + stage * BN_TM * BN_WS;
    unsigned* dr = sr + stage * BN_TN * BN_WS;
    for (int e = tid; e < BN_TM * 8; e += SP_THREADS) {
      const int v = e >> 3, h = e & 7, r = row0 + v;
      cpa16b(df + v * BN_WS + 4 * h, Bf + (int64_t)(r < nfit ? r : 0) * W + kc * BN_KW + 4 * h, r < nfit);
    }
    for (int e = tid; e < BN_TN * 8; e += SP_THREADS) {
      const int v = e >> 3, h = e & 7, j = tile * BN_TN + v;
      cpa16b(dr + v * BN_WS + 4 * h, Br + (int64_t)(j < nref ? j : 0) * W + kc * BN_KW + 4 * h, j < nref);
    }
  };
  for (int tile = 0; tile < ntiles; ++tile) {
    __syncthreads();
    if (tid < BN_TN) {
      const int j = tile * BN_TN + tid;
      scr[tid] = (j < nref) ? cr[j] : 0;
    }
    int acc[2][4];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = 0;
    load(0, tile, 0);
    asm volatile("cp.async.commit_group;\n" ::);
    for (int kc = 0; kc < nch; ++kc) {
      if (kc + 1 < nch) {
        load((kc + 1) & 1, tile, kc + 1);
        asm volatile("cp.async.commit_group;\n" ::);
        asm volatile("cp.async.wait_group 1;\n" ::);
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::);
      }
      __syncthreads();
      const unsigned* df = sf + (kc & 1) * BN_TM * BN_WS;
      const unsigned* dr = sr + (kc & 1) * BN_TN * BN_WS;
#pragma unroll
      for (int a = 0; a < BN_KW; a += 4) {
        uint4 fv[2], rv[4];
#pragma unroll
        for (int p = 0; p < 2; ++p) fv[p] = *reinterpret_cast<const uint4*>(df + (ty + 16 * p) * BN_WS + a);
#pragma unroll
        for (int q = 0; q < 4; ++q) rv[q] = *reinterpret_cast<const uint4*>(dr + (tx + 16 * q) * BN_WS + a);
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q)
            acc[p][q] += __popc(fv[p].x & rv[q].x) + __popc(fv[p].y & rv[q].y) + __popc(fv[p].z & rv[q].z) +
                         __popc(fv[p].w & rv[q].w);
      }
      __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const int lr = ty + 16 * p;
      if (row0 + lr >= nfit) continue;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = tile * BN_TN + tx + 16 * q;
        if (j >= nref) continue;
        const float s = (float)(cnt_f[p] + scr[tx + 16 * q] - 2 * acc[p][q]);  // exact below 2^24
        if (s < sthr[lr]) {
          const int pos = atomicAdd(&scnt[lr], 1);
          pool[lr * P2 + pos] = mds_pack_key(s, j);
        }
      }
    }
    __syncthreads();
    for (int r = warp; r < BN_TM; r += SP_THREADS / 32) {
      const int n = scnt[r];
      if (n <= k1) continue;
      warp_bitonic_sort(pool + r * P2, n, P2, lane);
      if (lane == 0) {
        scnt[r] = k1;
        sthr[r] = mds_key_value(pool[r * P2 + k1 - 1]);
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int r = warp; r < BN_TM; r += SP_THREADS / 32) {
    const int row = row0 + r;
    if (row >= nfit) continue;
    warp_bitonic_sort(pool + r * P2, scnt[r], P2, lane);
    for (int x = lane; x < k; x += 32) {
      const uint64_t key = pool[r * P2 + x + 1];
      out_d[(int64_t)row * k + x] = sqrt((double)mds_key_value(key));
      out_i[(int64_t)row * k + x] = mds_key_index(key);
    }
  }
}

static size_t bin_knn_smem(int k) {
  return sizeof(unsigned) * 2 * (BN_TM + BN_TN) * BN_WS + sizeof(int) * (BN_TN + BN_TM) + sizeof(float) * BN_TM +
         sizeof(uint64_t) * BN_TM * next_pow2(k + 1 + BN_TN) + 16;
}

// every value exactly 1.0 and every row's indices strictly ascending and >= 0
static bool binary_rows(const int64_t* off, const int32_t* idx, const double* val, int n, int* dmax) {
  for (int r = 0; r < n; ++r)
    for (int64_t e = off[r]; e < off[r + 1]; ++e) {
      if (val[e] != 1.0 || idx[e] < 0 || (e > off[r] && idx[e] <= idx[e - 1])) return false;
      *dmax = std::max(*dmax, idx[e]);
    }
  return true;
}

// ---------------------------------------------------------------------------
// contact_profile
// ---------------------------------------------------------------------------
// distance(a, b) * 10 < eps exactly as the reference decides it
__device__ __forceinline__ bool contact_exact(const float* a, const float* b, double eps) {
  double d = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float t = __fsub_rn(a[c], b[c]);
    d = __dadd_rn(d, (double)__fmul_rn(t, t));
  }
  return __dmul_rn(__dsqrt_rn(d), 10.0) < eps;
}
__device__ __forceinline__ bool contact_of(const float* a, const float* b, double eps, float eps_lo, float eps_hi) {
  const float t0 = a[0] - b[0], t1 = a[1] - b[1], t2 = a[2] - b[2];
  const float d = sqrtf(fmaf(t0, t0, fmaf(t1, t1, t2 * t2))) * 10.0f;  // within ~1e-6 relative
  if (d < eps_lo) return true;
  if (d > eps_hi) return false;
  return contact_exact(a, b, eps);
}

// mode 0: count each frame's contacts into counts[f]; mode 1: write them in
// ascending grid order at idx[offsets[f] ...]. One block per frame.
__global__ void __launch_bounds__(SP_THREADS)
k_contact(const float* __restrict__ xyz, int natoms, const int* __restrict__ g1, int n1, const int* __restrict__ g2,
          int n2, double eps, int mode, int64_t* __restrict__ counts, const int64_t* __restrict__ offsets,
          int* __restrict__ idx) {
  __shared__ int wsum[SP_THREADS / 32];
  __shared__ int64_t s_base;
  const int f = blockIdx.x;
  const float* x = xyz + (int64_t)f * natoms * 3;
  const float eps_lo = (float)(eps * (1.0 - 1e-5)), eps_hi = (float)(eps * (1.0 + 1e-5));
  const int64_t total = (int64_t)n1 * n2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = (mode == 1) ? offsets[f] : 0;
  int64_t mine = 0;
  __syncthreads();
  for (int64_t p0 = 0; p0 < total; p0 += blockDim.x) {
    const int64_t p = p0 + threadIdx.x;
    bool hit = false;
    if (p < total) {
      const int i = (int)(p / n2), j = (int)(p % n2);
      const float* a = x + 3 * (int64_t)g1[i];
      const float* b = x + 3 * (int64_t)g2[j];
      const float av[3] = {a[0], a[1], a[2]}, bv[3] = {b[0], b[1], b[2]};
      hit = contact_of(av, bv, eps, eps_lo, eps_hi);
    }
    if (mode == 0) {
      mine += hit ? 1 : 0;
      continue;
    }
    // ordered compaction of this chunk: warp ballots, then warp offsets
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int before = 0, chunk = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      before += (w < warp) ? wsum[w] : 0;
      chunk += wsum[w];
    }
    if (hit) idx[s_base + before + __popc(bal & ((1u << lane) - 1u))] = (int)p;
    __syncthreads();
    if (threadIdx.x == 0) s_base += chunk;
    __syncthreads();
  }
  if (mode == 0) {
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
    if (lane == 0) wsum[warp] = (int)mine;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
      counts[f] = t;
    }
  }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int mds_knn_data_sparse(mds_ctx* ctx, const int64_t* ref_off, const int32_t* ref_idx,
                                   const double* ref_val, int n_ref, const int64_t* fit_off, const int32_t* fit_idx,
                                   const double* fit_val, int n_fit, int k, unsigned flags, double* out_d,
                                   int32_t* out_i, int* k_used) {
  if (!ctx) return MDS_ERR_ARG;
  ctx->stats = mds_knn_stats{};
  if (!ref_off || !out_d || !out_i || (n_ref > 0 && (!ref_idx || !ref_val)))
    return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  if (n_ref < 1 || n_fit < 0) return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes: n_ref=%d n_fit=%d", n_ref, n_fit);
  const bool full = (flags & MDS_FULL) != 0;
  const bool same = (fit_off == nullptr);
  if (same) {
    fit_off = ref_off;
    fit_idx = ref_idx;
    fit_val = ref_val;
    n_fit = n_ref;
  }
  // knn_data_sparse.cpp:199-202: k clamped to N_ref - 1
  if (!full) {
    if (k < 0) return mds_fail(ctx, MDS_ERR_ARG, "k must be >= 0");
    if (n_ref - 1 < k) k = n_ref - 1;
    if (k + 1 > 2048) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d exceeds the supported maximum of 2047", k);
  }
  if (k_used) *k_used = k;
  ctx->stats.pairs = (long long)n_ref * n_fit;
  if (n_fit == 0 || (!full && k == 0)) return MDS_OK;
  const int64_t nnz_r = ref_off[n_ref], nnz_f = fit_off[n_fit];
  if (ref_off[0] != 0 || nnz_r < 0 || fit_off[0] != 0 || nnz_f < 0)
    return mds_fail(ctx, MDS_ERR_ARG, "offsets must start at 0 and be non-decreasing");
  for (int r = 0; r < n_ref; ++r)
    if (ref_off[r + 1] < ref_off[r]) return mds_fail(ctx, MDS_ERR_ARG, "reference offsets decrease at row %d", r);
  if (!same)
    for (int r = 0; r < n_fit; ++r)
      if (fit_off[r + 1] < fit_off[r]) return mds_fail(ctx, MDS_ERR_ARG, "fit offsets decrease at row %d", r);
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const int mode = full ? 1 : 0;
  const size_t width = full ? (size_t)n_ref : (size_t)k;
  DevBuf dro(ctx), dri(ctx), drv(ctx), dfo(ctx), dfi(ctx), dfv(ctx), dd(ctx), di(ctx);
  MDS_TRY(dro.alloc(ctx, sizeof(int64_t) * (n_ref + 1)));
  MDS_TRY(dri.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz_r, 1)));
  MDS_TRY(drv.alloc(ctx, sizeof(double) * std::max<int64_t>(nnz_r, 1)));
  MDS_CUDA(ctx, cudaMemcpyAsync(dro.p, ref_off, sizeof(int64_t) * (n_ref + 1), cudaMemcpyHostToDevice, s));
  if (nnz_r) {
    MDS_CUDA(ctx, cudaMemcpyAsync(dri.p, ref_idx, sizeof(int) * nnz_r, cudaMemcpyHostToDevice, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(drv.p, ref_val, sizeof(double) * nnz_r, cudaMemcpyHostToDevice, s));
  }
  const int64_t* pfo = dro.as<int64_t>();
  const int* pfi = dri.as<int>();
  const double* pfv = drv.as<double>();
  if (!same) {
    MDS_TRY(dfo.alloc(ctx, sizeof(int64_t) * (n_fit + 1)));
    MDS_TRY(dfi.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz_f, 1)));
    MDS_TRY(dfv.alloc(ctx, sizeof(double) * std::max<int64_t>(nnz_f, 1)));
    MDS_CUDA(ctx, cudaMemcpyAsync(dfo.p, fit_off, sizeof(int64_t) * (n_fit + 1), cudaMemcpyHostToDevice, s));
    if (nnz_f) {
      MDS_CUDA(ctx, cudaMemcpyAsync(dfi.p, fit_idx, sizeof(int) * nnz_f, cudaMemcpyHostToDevice, s));
      MDS_CUDA(ctx, cudaMemcpyAsync(dfv.p, fit_val, sizeof(double) * nnz_f, cudaMemcpyHostToDevice, s));
    }
    pfo = dfo.as<int64_t>();
    pfi = dfi.as<int>();
    pfv = dfv.as<double>();
  }
  MDS_TRY(dd.alloc(ctx, sizeof(double) * width * n_fit));
  MDS_TRY(di.alloc(ctx, sizeof(int) * width * n_fit));
  // binary vectors: bit sets and popcount tiles (exact, no walk per pair)
  int dmax = -1;
  const bool binary = !full && binary_rows(ref_off, ref_idx, ref_val, n_ref, &dmax) &&
                      (same || binary_rows(fit_off, fit_idx, fit_val, n_fit, &dmax)) && dmax < (1 << 24) - 1;
  const int W = mds_round_up(std::max(dmax + 1, 1), 32 * BN_KW) / 32;
  if (binary && (size_t)W * 4 * ((size_t)n_ref + (same ? 0 : n_fit)) <= ((size_t)8 << 30)) {
    DevBuf br(ctx), bf(ctx), cr(ctx), cf(ctx);
    MDS_TRY(br.alloc(ctx, sizeof(unsigned) * (size_t)W * n_ref));
    MDS_TRY(cr.alloc(ctx, sizeof(int) * n_ref));
    MDS_CUDA(ctx, cudaMemsetAsync(br.p, 0, sizeof(unsigned) * (size_t)W * n_ref, s));
    std::vector<int> hc(std::max(n_ref, n_fit));
    for (int r = 0; r < n_ref; ++r) hc[r] = (int)(ref_off[r + 1] - ref_off[r]);
    MDS_CUDA(ctx, cudaMemcpyAsync(cr.p, hc.data(), sizeof(int) * n_ref, cudaMemcpyHostToDevice, s));
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    k_bitset<<<n_ref, 128, 0, s>>>(dro.as<int64_t>(), dri.as<int>(), W, br.as<unsigned>());
    const unsigned* pbf = br.as<unsigned>();
    const int* pcf = cr.as<int>();
    if (!same) {
      MDS_TRY(bf.alloc(ctx, sizeof(unsigned) * (size_t)W * n_fit));
      MDS_TRY(cf.alloc(ctx, sizeof(int) * n_fit));
      MDS_CUDA(ctx, cudaMemsetAsync(bf.p, 0, sizeof(unsigned) * (size_t)W * n_fit, s));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));  // hc is reused
      for (int r = 0; r < n_fit; ++r) hc[r] = (int)(fit_off[r + 1] - fit_off[r]);
      MDS_CUDA(ctx, cudaMemcpyAsync(cf.p, hc.data(), sizeof(int) * n_fit, cudaMemcpyHostToDevice, s));
      k_bitset<<<n_fit, 128, 0, s>>>(pfo, pfi, W, bf.as<unsigned>());
      pbf = bf.as<unsigned>();
      pcf = cf.as<int>();
    }
    MDS_CUDA(ctx, cudaGetLastError());
    const size_t bsm = bin_knn_smem(k);
    static bool bin_done = false;
    static size_t bin_limit = 0;
    MDS_TRY(mds_allow_dyn_smem(ctx, k_bin_knn, &bin_done, &bin_limit));
    if (bsm > bin_limit) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d too large", k);
    ctx->stats.launches = same ? 2 : 3;
    k_bin_knn<<<(n_fit + BN_TM - 1) / BN_TM, SP_THREADS, bsm, s>>>(pbf, pcf, n_fit, br.as<unsigned>(), cr.as<int>(),
                                                                    n_ref, W, k, dd.as<double>(), di.as<int>());
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    MDS_CUDA(ctx, cudaMemcpyAsync(out_d, dd.p, sizeof(double) * width * n_fit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(out_i, di.p, sizeof(int) * width * n_fit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    ctx->stats.screen_ms = ms;
    ctx->stats.passes = 1;
    return MDS_OK;
  }
  const size_t smem = sparse_knn_smem(k, mode);
  static bool attr_done = false;
  static size_t attr_limit = 0;
  MDS_TRY(mds_allow_dyn_smem(ctx, k_sparse_knn, &attr_done, &attr_limit));
  if (smem > attr_limit) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k=%d too large", k);
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  ctx->stats.launches = 1;
  k_sparse_knn<<<n_fit, SP_THREADS, smem, s>>>(dro.as<int64_t>(), dri.as<int>(), drv.as<double>(), n_ref, pfo, pfi,
                                               pfv, k, mode, dd.as<double>(), di.as<int>());
  MDS_CUDA(ctx, cudaGetLastError());
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  MDS_CUDA(ctx, cudaMemcpyAsync(out_d, dd.p, sizeof(double) * width * n_fit, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(out_i, di.p, sizeof(int) * width * n_fit, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
  ctx->stats.recheck_ms = ms;
  ctx->stats.passes = 1;
  return MDS_OK;
}

extern "C" int mds_contact_profile(mds_ctx* ctx, const float* xyz, int nframes, int natoms, const int32_t* g1, int n1,
                                   const int32_t* g2, int n2, double eps, int64_t* offsets, int32_t* idx,
                                   int64_t idx_cap) {
  if (!ctx) return MDS_ERR_ARG;
  if (!xyz || !g1 || !g2 || !offsets) return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  if (nframes < 0 || natoms < 1 || n1 < 1 || n2 < 1)
    return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes: nframes=%d natoms=%d n1=%d n2=%d", nframes, natoms, n1, n2);
  if ((int64_t)n1 * n2 > 0x7fffffff) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "grid of %d x %d pairs", n1, n2);
  for (int i = 0; i < n1; ++i)
    if (g1[i] < 0 || g1[i] >= natoms) return mds_fail(ctx, MDS_ERR_ARG, "group 1 atom %d out of range", g1[i]);
  for (int j = 0; j < n2; ++j)
    if (g2[j] < 0 || g2[j] >= natoms) return mds_fail(ctx, MDS_ERR_ARG, "group 2 atom %d out of range", g2[j]);
  offsets[0] = 0;
  if (nframes == 0) return MDS_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  DevBuf dx(ctx), dg1(ctx), dg2(ctx), dcnt(ctx), doff(ctx), didx(ctx);
  const size_t xbytes = sizeof(float) * 3 * (size_t)natoms * nframes;
  MDS_TRY(dx.alloc(ctx, xbytes));
  MDS_TRY(dg1.alloc(ctx, sizeof(int) * n1));
  MDS_TRY(dg2.alloc(ctx, sizeof(int) * n2));
  MDS_TRY(dcnt.alloc(ctx, sizeof(int64_t) * nframes));
  MDS_CUDA(ctx, cudaMemcpyAsync(dx.p, xyz, xbytes, cudaMemcpyHostToDevice, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(dg1.p, g1, sizeof(int) * n1, cudaMemcpyHostToDevice, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(dg2.p, g2, sizeof(int) * n2, cudaMemcpyHostToDevice, s));
  k_contact<<<nframes, SP_THREADS, 0, s>>>(dx.as<float>(), natoms, dg1.as<int>(), n1, dg2.as<int>(), n2, eps, 0,
                                           dcnt.as<int64_t>(), nullptr, nullptr);
  MDS_CUDA(ctx, cudaGetLastError());
  std::vector<int64_t> cnt(nframes);
  MDS_CUDA(ctx, cudaMemcpyAsync(cnt.data(), dcnt.p, sizeof(int64_t) * nframes, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  for (int f = 0; f < nframes; ++f) offsets[f + 1] = offsets[f] + cnt[f];
  const int64_t total = offsets[nframes];
  if (!idx) return MDS_OK;
  if (idx_cap < total)
    return mds_fail(ctx, MDS_ERR_ARG, "index buffer holds %lld entries, %lld needed", (long long)idx_cap,
                    (long long)total);
  if (total == 0) return MDS_OK;
  MDS_TRY(doff.alloc(ctx, sizeof(int64_t) * (nframes + 1)));
  MDS_TRY(didx.alloc(ctx, sizeof(int) * total));
  MDS_CUDA(ctx, cudaMemcpyAsync(doff.p, offsets, sizeof(int64_t) * (nframes + 1), cudaMemcpyHostToDevice, s));
  k_contact<<<nframes, SP_THREADS, 0, s>>>(dx.as<float>(), natoms, dg1.as<int>(), n1, dg2.as<int>(), n2, eps, 1,
                                           nullptr, doff.as<int64_t>(), didx.as<int>());
  MDS_CUDA(ctx, cudaGetLastError());
  MDS_CUDA(ctx, cudaMemcpyAsync(idx, didx.p, sizeof(int) * total, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  return MDS_OK;
}
