// knn_data.cu -- k nearest vectors (knn_data) on sm_103a.
//
// Replaces the compute core of knn_data.cpp:176-250 with
// euclidean_distance (mdsctk.cpp:330-335) or correlation_distance
// (mdsctk.cpp:337-360).
//
//  1. k_vec_prep   per vector: FP32 copy (screen operand), squared norm, and
//                  for the correlation metric the reference's own sums in its
//                  order (sum, sum of squares -> mean and scale) and the
//                  standardized FP32 vector.
//  2. k_screen_dot all pairs: FP32 dot products on CUDA cores (64 x 64 tile,
//                  4 x 4 pairs per thread), screen value = lower bound of the
//                  squared distance (Euclidean: |x|^2 + |y|^2 - 2 x.y, minus a
//                  rounding guard; correlation: (1 - r)/2 minus a guard),
//                  fused per-row top-K' in shared memory.
//  3. k_data_recheck merge the column segments, recompute every candidate in
//                  FP64 with the reference's exact operation order (no fused
//                  multiply-add, sequential sum), select k+1 by (value, index),
//                  drop position 0, verify the guard.
#include <algorithm>
#include <mutex>
#include <cmath>
#include <vector>

#include "knn_common.cuh"
#include "warp_sort.cuh"

#define DT_TM 64
#define DT_TN 64
#define DT_KC 32
#define DT_THREADS 256
#define DT_FS 36  // floats per vector per stage (32 + 4: bank spread, 16-byte rows)
#define DT_MAX_KP 192  // largest K' whose pools (64 rows x (K' + 64) keys) fit in shared memory

// ---------------------------------------------------------------------------
// 1. per-vector preparation
// ---------------------------------------------------------------------------
// X [n][dim] double -> Xf [n][Dp] float (plain or standardized), nrm[n]
// (float squared norm of the screen operand), mean/scale (double, for the
// correlation recheck).
__global__ void k_vec_prep(const double* __restrict__ X, int n, int dim, int Dp, int corr,
                           float* __restrict__ Xf, float* __restrict__ nrm, double* __restrict__ mean,
                           double* __restrict__ scale) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double* x = X + (int64_t)v * dim;
  float* o = Xf + (int64_t)v * Dp;
  if (!corr) {
    float s = 0.f;
    for (int i = 0; i < dim; ++i) {
      float f = (float)x[i];
      o[i] = f;
      s = fmaf(f, f, s);
    }
    for (int i = dim; i < Dp; ++i) o[i] = 0.f;
    nrm[v] = s;
    return;
  }
  // the reference's single-pass sums (correlation_distance, mdsctk.cpp:339-351)
  double sum = 0.0, sq = 0.0, dsize = (double)dim;
  for (int i = 0; i < dim; ++i) {
    sum = __dadd_rn(sum, x[i]);
    sq = __dadd_rn(sq, __dmul_rn(x[i], x[i]));
  }
  double sd = sqrt(__ddiv_rn(__dsub_rn(__dmul_rn(dsize, sq), __dmul_rn(sum, sum)),
                             __dmul_rn(dsize, __dsub_rn(dsize, 1.0))));
  double mu = __ddiv_rn(sum, dsize);
  mean[v] = mu;
  scale[v] = sd;
  // standardized screen operand: z = (x - mean) / (sd * sqrt(dim - 1)), so r = z_a . z_b
  double inv = (sd > 0.0) ? 1.0 / (sd * sqrt(dsize - 1.0)) : 0.0;
  float s = 0.f;
  for (int i = 0; i < dim; ++i) {
    float f = (float)((x[i] - mu) * inv);
    o[i] = f;
    s = fmaf(f, f, s);
  }
  for (int i = dim; i < Dp; ++i) o[i] = 0.f;
  nrm[v] = s;
}

// ---------------------------------------------------------------------------
// 2. screen
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cpa16(void* smem, const void* gmem, bool valid) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}

__global__ void __launch_bounds__(DT_THREADS, 1)
k_screen_dot(const float* __restrict__ Xf, const float* __restrict__ Xr, const float* __restrict__ nf,
             const float* __restrict__ nr, int nrows, const int* __restrict__ rowlist, int Nr, int Dp,
             int corr, float guard, int Kp, int nseg, uint64_t* __restrict__ cand, int* __restrict__ cand_n) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sf = reinterpret_cast<float*>(smem_raw);        // [2][64*36]
  float* sr = sf + 2 * DT_TM * DT_FS;                     // [2][64*36]
  float* snr = sr + 2 * DT_TN * DT_FS;                    // [64]
  int* scnt = reinterpret_cast<int*>(snr + DT_TN);        // [64]
  float* sthr = reinterpret_cast<float*>(scnt + DT_TM);   // [64]
  uint64_t* pool = reinterpret_cast<uint64_t*>(sthr + DT_TM);
  const int P2 = next_pow2(Kp + DT_TN);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, lane = tid & 31, warp = tid >> 5;
  const int rt = blockIdx.x / nseg, seg = blockIdx.x % nseg;
  const int row0 = rt * DT_TM;
  const int ntiles = (Nr + DT_TN - 1) / DT_TN;
  const int t0 = (int)((int64_t)ntiles * seg / nseg), t1 = (int)((int64_t)ntiles * (seg + 1) / nseg);
  int grow[4];
  float rn[4];
  for (int p = 0; p < 4; ++p) {
    int lr = row0 + ty + 16 * p;
    grow[p] = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
    rn[p] = grow[p] >= 0 ? nf[grow[p]] : 0.f;
  }
  if (tid < DT_TM) {
    scnt[tid] = 0;
    sthr[tid] = __int_as_float(0x7f800000);
  }
  const int nch = Dp / DT_KC;
  auto load = [&](int stage, int tile, int kc) {
    float* df = sf + stage * DT_TM * DT_FS;
    float* dr = sr + stage * DT_TN * DT_FS;
    for (int e = tid; e < DT_TM * 8; e += DT_THREADS) {
      int v = e >> 3, h = e & 7;
      int lr = row0 + v;
      int g = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
      cpa16(df + v * DT_FS + 4 * h, Xf + (int64_t)(g < 0 ? 0 : g) * Dp + kc * DT_KC + 4 * h, g >= 0);
    }
    for (int e = tid; e < DT_TN * 8; e += DT_THREADS) {
      int v = e >> 3, h = e & 7;
      int j = tile * DT_TN + v;
      cpa16(dr + v * DT_FS + 4 * h, Xr + (int64_t)(j < Nr ? j : 0) * Dp + kc * DT_KC + 4 * h, j < Nr);
    }
  };
  for (int tile = t0; tile < t1; ++tile) {
    __syncthreads();
    if (tid < DT_TN) {
      int j = tile * DT_TN + tid;
      snr[tid] = (j < Nr) ? nr[j] : 0.f;
    }
    float acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
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
      const float* df = sf + (kc & 1) * DT_TM * DT_FS;
      const float* dr = sr + (kc & 1) * DT_TN * DT_FS;
#pragma unroll
      for (int a = 0; a < DT_KC; a += 4) {
        float4 fv[4], rv[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) fv[p] = *reinterpret_cast<const float4*>(df + (ty + 16 * p) * DT_FS + a);
#pragma unroll
        for (int q = 0; q < 4; ++q) rv[q] = *reinterpret_cast<const float4*>(dr + (tx + 16 * q) * DT_FS + a);
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            acc[p][q] = fmaf(fv[p].x, rv[q].x, acc[p][q]);
            acc[p][q] = fmaf(fv[p].y, rv[q].y, acc[p][q]);
            acc[p][q] = fmaf(fv[p].z, rv[q].z, acc[p][q]);
            acc[p][q] = fmaf(fv[p].w, rv[q].w, acc[p][q]);
          }
      }
      __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (grow[p] < 0) continue;
      int lr = ty + 16 * p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int j = tile * DT_TN + tx + 16 * q;
        if (j >= Nr) continue;
        float cn = snr[tx + 16 * q];
        float s = corr ? 0.5f * (1.0f - acc[p][q]) : rn[p] + cn - 2.0f * acc[p][q];
        s = fmaxf(s - guard * (rn[p] + cn), 0.0f);
        if (s < sthr[lr]) {
          int pos = atomicAdd(&scnt[lr], 1);
          pool[lr * P2 + pos] = mds_pack_key(s, j);
        }
      }
    }
    __syncthreads();
    for (int r = warp; r < DT_TM; r += DT_THREADS / 32) {
      int n = scnt[r];
      if (n <= Kp) continue;
      warp_bitonic_sort(pool + r * P2, n, P2, lane);
      if (lane == 0) {
        scnt[r] = Kp;
        sthr[r] = mds_key_value(pool[r * P2 + Kp - 1]);
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int r = warp; r < DT_TM; r += DT_THREADS / 32) {
    int lr = row0 + r;
    if (lr >= nrows) continue;
    int n = min(scnt[r], Kp);
    warp_bitonic_sort(pool + r * P2, scnt[r], P2, lane);
    uint64_t* dst = cand + ((int64_t)lr * nseg + seg) * Kp;
    for (int x = lane; x < n; x += 32) dst[x] = pool[r * P2 + x];
    if (lane == 0) cand_n[(int64_t)lr * nseg + seg] = n;
  }
}

static size_t screen_dot_smem(int Kp) {
  return sizeof(float) * (2 * DT_TM * DT_FS + 2 * DT_TN * DT_FS + DT_TN) + sizeof(int) * DT_TM +
         sizeof(float) * DT_TM + sizeof(uint64_t) * DT_TM * next_pow2(Kp + DT_TN);
}

// ---------------------------------------------------------------------------
// 3. exact recheck in the reference's arithmetic
// ---------------------------------------------------------------------------
// euclidean_distance(size, reference=fit row a, fitting=ref row b)
__device__ __forceinline__ double exact_euclid(const double* a, const double* b, int dim) {
  double value = 0.0;
  for (int x = 0; x < dim; ++x) {
    double t = __dsub_rn(a[x], b[x]);
    value = __dadd_rn(value, __dmul_rn(t, t));
  }
  return value;  // squared; sqrt taken by the caller
}
// correlation_distance with per-vector means/scales precomputed by k_vec_prep
__device__ __forceinline__ double exact_corr(const double* a, double ma, double sa, const double* b, double mb,
                                             double sb, int dim) {
  double dsize = (double)dim, value = 0.0;
  for (int x = 0; x < dim; ++x) value = __dadd_rn(value, __dmul_rn(__dsub_rn(a[x], ma), __dsub_rn(b[x], mb)));
  value = __ddiv_rn(__dsub_rn(1.0, __ddiv_rn(value, __dmul_rn(__dmul_rn(__dsub_rn(dsize, 1.0), sa), sb))), 2.0);
  if (value < 0.0) value = 0.0;
  return value;  // squared distance; sqrt taken by the caller
}

// the same on vectors already centred (x - mean, in the reference's own
// subtraction, by k_vec_center): the products and sums are unchanged
__device__ __forceinline__ double exact_corr_centred(const double* ac, double sa, const double* bc, double sb,
                                                     int dim) {
  double dsize = (double)dim, value = 0.0;
  for (int x = 0; x < dim; ++x) value = __dadd_rn(value, __dmul_rn(ac[x], bc[x]));
  value = __ddiv_rn(__dsub_rn(1.0, __ddiv_rn(value, __dmul_rn(__dmul_rn(__dsub_rn(dsize, 1.0), sa), sb))), 2.0);
  if (value < 0.0) value = 0.0;
  return value;
}

// Xc [n][dim] = X - mean of its vector, for the correlation recheck: each
// (x - mean) of correlation_distance (mdsctk.cpp:349) is a per-vector
// value, computed once here instead of once per pair.
__global__ void k_vec_center(const double* __restrict__ X, int64_t total, int dim, const double* __restrict__ mean,
                             double* __restrict__ Xc) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    Xc[e] = __dsub_rn(X[e], mean[e / dim]);
}

#define DR_THREADS 256

// One block per fit row. mode 0: candidates from the screen; mode 1: every
// reference (exact row); mode 2: full row output in reference order.
__global__ void __launch_bounds__(DR_THREADS)
k_data_recheck(const double* __restrict__ Xfit, const double* __restrict__ Xref, const double* __restrict__ mf,
               const double* __restrict__ sfv, const double* __restrict__ mr, const double* __restrict__ srv,
               const float* __restrict__ nf, int nrows, const int* __restrict__ rowlist, int Nr, int dim, int corr,
               int mode, const uint64_t* __restrict__ cand, const int* __restrict__ cand_n, int nseg, int Kp, int k,
               const float* __restrict__ rowthr, double* __restrict__ out_d, int* __restrict__ out_i,
               int* __restrict__ flagged, int* __restrict__ nflag, int cand_by_row) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* sa = reinterpret_cast<double*>(smem_raw);              // [dim]
  uint64_t* keys = reinterpret_cast<uint64_t*>(sa + dim);        // merge buffer, then candidates
  __shared__ int s_total;
  const int lr = blockIdx.x;
  if (lr >= nrows) return;
  const int grow = rowlist ? rowlist[lr] : lr;
  for (int e = threadIdx.x; e < dim; e += blockDim.x) sa[e] = Xfit[(int64_t)grow * dim + e];
  const double ma = corr ? mf[grow] : 0.0, sda = corr ? sfv[grow] : 0.0;
  const int k1 = k + 1;
  __syncthreads();
  if (mode == 2) {
    for (int j = threadIdx.x; j < Nr; j += blockDim.x) {
      const double* b = Xref + (int64_t)j * dim;
      double v = corr ? exact_corr(sa, ma, sda, b, mr[j], srv[j], dim) : exact_euclid(sa, b, dim);
      out_d[(int64_t)grow * Nr + j] = sqrt(v);
      out_i[(int64_t)grow * Nr + j] = j;
    }
    return;
  }
  int total;
  float tau = __int_as_float(0x7f800000);
  const int crow = cand_by_row ? grow : lr;  // candidate lists by fit row or by position in rowlist
  if (mode == 0) {
    if (threadIdx.x == 0) {
      int t = 0;
      for (int s = 0; s < nseg; ++s) t += cand_n[(int64_t)crow * nseg + s];
      s_total = t;
    }
    __syncthreads();
    const int t = s_total;
    const int P2 = next_pow2(max(t, 1));
    int off = 0;
    for (int s = 0; s < nseg; ++s) {
      int ns = cand_n[(int64_t)crow * nseg + s];
      const uint64_t* src = cand + ((int64_t)crow * nseg + s) * Kp;
      for (int x = threadIdx.x; x < ns; x += blockDim.x) keys[off + x] = src[x];
      off += ns;
    }
    for (int x = t + threadIdx.x; x < P2; x += blockDim.x) keys[x] = MDS_KEY_INF;
    __syncthreads();
    block_bitonic_sort(keys, P2);
    total = min(t, Kp);
    // the bound of every pair left out: the K'-th candidate's, or the
    // threshold the screen filtered them with, whichever is smaller (the
    // tensor-core screen's thresholds follow the (k+1)-th bound, so its
    // final threshold can lie below the K'-th candidate)
    if (t >= Kp) tau = mds_key_value(keys[Kp - 1]);
    if (rowthr) tau = fminf(tau, rowthr[grow]);
  } else {
    total = Nr;
  }
  // Exact (value, index) pairs: the k+1 best so far in slots [0, k1), the
  // chunk being rechecked after them; the candidate keys stay in keys[0, Kp).
  const int CH = (mode == 0) ? next_pow2(max(Kp, 1)) : 1024;
  const int BP2 = next_pow2(k1 + CH);
  double* bval = reinterpret_cast<double*>(keys + (mode == 0 ? Kp : 0));
  int* bidx = reinterpret_cast<int*>(bval + BP2);
  // mode 0: candidates in order of their bound; the first k+1 + k/4 are
  // rechecked, the rest only if the next bound is not above the (k+1)-th
  // exact value so far, or that value is not below tau (otherwise nothing
  // later, and no pair left out, can enter the k+1 best)
  const int first = (mode == 0) ? min(max(total, 1), k1 + max(8, k1 / 4)) : CH;
  __shared__ int s_stop;
  bool stopped = false;
  for (int x = threadIdx.x; x < BP2; x += blockDim.x) {
    bval[x] = __longlong_as_double(0x7ff0000000000000ll);
    bidx[x] = 0x7fffffff;
  }
  __syncthreads();
  for (int base = 0; base < total;) {
    const int nc = (mode == 0) ? (base == 0 ? first : total - base) : min(CH, total - base);
    for (int c = threadIdx.x; c < BP2 - k1; c += blockDim.x) {
      double v = __longlong_as_double(0x7ff0000000000000ll);
      int j = 0x7fffffff;
      if (c < nc) {
        j = (mode == 0) ? mds_key_index(keys[base + c]) : base + c;
        const double* b = Xref + (int64_t)j * dim;
        v = corr ? exact_corr(sa, ma, sda, b, mr[j], srv[j], dim) : exact_euclid(sa, b, dim);
      }
      bval[k1 + c] = v;
      bidx[k1 + c] = j;
    }
    __syncthreads();
    // bitonic sort of (value, index) pairs
    for (int kk = 2; kk <= BP2; kk <<= 1)
      for (int jj = kk >> 1; jj > 0; jj >>= 1) {
        for (int i = threadIdx.x; i < BP2; i += blockDim.x) {
          int ixj = i ^ jj;
          if (ixj > i) {
            double va = bval[i], vb = bval[ixj];
            int ia = bidx[i], ib = bidx[ixj];
            // the values are non-negative (or +inf): their bit patterns order
            // as unsigned integers, so the compare stays off the FP64 pipe
            const unsigned long long ua = __double_as_longlong(va), ub = __double_as_longlong(vb);
            bool gt = (ua > ub) || (ua == ub && ia > ib);
            bool up = (i & kk) == 0;
            if (gt == up) {
              bval[i] = vb; bval[ixj] = va;
              bidx[i] = ib; bidx[ixj] = ia;
            }
          }
        }
        __syncthreads();
      }
    base += nc;
    if (mode == 0 && base < total) {
      if (threadIdx.x == 0)
        s_stop = (bval[k1 - 1] < (double)mds_key_value(keys[base]) && bval[k1 - 1] < (double)tau) ? 1 : 0;
      __syncthreads();
      if (s_stop) {
        stopped = true;
        break;
      }
    }
  }
  if (threadIdx.x == 0 && mode == 0 && !stopped) {
    // strict: a pair left out of the list has a lower bound >= tau, so only
    // dk < tau proves that no left-out pair ties with or beats the k+1-th
    double dk = bval[k1 - 1];
    if (!(dk < (double)tau)) {
      int pos = atomicAdd(nflag, 1);
      flagged[pos] = grow;
    }
  }
  for (int x = threadIdx.x; x < k; x += blockDim.x) {
    out_d[(int64_t)grow * k + x] = sqrt(bval[x + 1]);
    out_i[(int64_t)grow * k + x] = bidx[x + 1];
  }
}

// ---------------------------------------------------------------------------
// 3b. the candidate recheck (mode 0) in three stages
// ---------------------------------------------------------------------------
// The same result as k_data_recheck mode 0, with no block-wide barrier and
// the FP64 work packed densely: keys and (value, index) pairs are sorted in
// registers by bitonic networks over a warp (element e = 32 i + lane). The
// first k + 3 candidates of each row are rechecked; rows that need more, or
// that hold more than RW_MAXT candidates, are listed in big[] for
// k_data_recheck. Used for k + 1 <= RW_MAXK1.
#define RW_WARPS 8
#define RW_MAXT 512   // merged candidates a warp sorts in registers
#define RW_MAXK1 64   // k + 1 (the first batch, k + 3, fits the finishing sort of 128)

// (value bits, index) pairs in ascending (value, index) order; the values
// are non-negative or +inf, so their bits order as unsigned integers
__device__ __forceinline__ bool pair_less(uint64_t a, int ia, uint64_t b, int ib) {
  return a < b || (a == b && ia < ib);
}
template <int PER>
__device__ __forceinline__ void wsort_pair(uint64_t (&v)[PER], int (&x)[PER], int lane) {
#pragma unroll
  for (int k = 2; k <= 32 * PER; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int p = i ^ (j >> 5);
          if (p > i) {
            const bool up = ((i * 32 + lane) & k) == 0;
            if (pair_less(v[p], x[p], v[i], x[i]) == up) {
              const uint64_t tv = v[i];
              const int tx = x[i];
              v[i] = v[p];
              x[i] = x[p];
              v[p] = tv;
              x[p] = tx;
            }
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int e = i * 32 + lane;
          const uint64_t ov = __shfl_xor_sync(0xffffffffu, v[i], j);
          const int ox = __shfl_xor_sync(0xffffffffu, x[i], j);
          const bool keepmin = ((e & j) == 0) == ((e & k) == 0);
          if (pair_less(ov, ox, v[i], x[i]) == keepmin) {
            v[i] = ov;
            x[i] = ox;
          }
        }
      }
    }
  }
}

// Stage 1, one warp per fit row: merge the segments' lists, sort the keys
// (element e < t comes from the segment s with off[s] <= e < off[s] + n[s]),
// and write the first `first` candidate indices in order of their bound
// (cidx [row][fw]), with the row's candidate count, tau (the bound of every
// pair left out: the K'-th candidate's, or the screen's threshold, whichever
// is smaller) and the next candidate's bound.
template <int PER>
__device__ void cands_row(const uint64_t* __restrict__ cand, int row, int nseg, int Kp, int k1, int fw, int t,
                          int segoff, int segn, float rthr, int* __restrict__ cidx, int4* __restrict__ meta,
                          int lane) {
  uint64_t v[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = i * 32 + lane;
    uint64_t key = MDS_KEY_INF;
    for (int s = 0; s < nseg; ++s) {
      const int o = __shfl_sync(0xffffffffu, segoff, s), nn = __shfl_sync(0xffffffffu, segn, s);
      if (e >= o && e < o + nn) key = cand[((int64_t)row * nseg + s) * Kp + (e - o)];
    }
    v[i] = key;
  }
  wsort_u64<PER>(v, lane);
  const int total = min(t, Kp);
  float tau = rthr;
  if (t >= Kp) tau = fminf(tau, mds_key_value(lane_elem<PER>(v, Kp - 1)));
  const int first = min(total, fw);
  const float nxt = (first < total) ? mds_key_value(lane_elem<PER>(v, first)) : __int_as_float(0x7f800000);
  for (int base = 0; base < fw; base += 32) {
    const int e = base + lane;
    const uint64_t key = lane_elem<PER>(v, min(e, 32 * PER - 1));
    if (e < first) cidx[(int64_t)row * fw + e] = mds_key_index(key);
  }
  if (lane == 0) meta[row] = make_int4(first, total, __float_as_int(tau), __float_as_int(nxt));
}

__global__ void __launch_bounds__(RW_WARPS * 32)
k_recheck_cands(const uint64_t* __restrict__ cand, const int* __restrict__ cand_n, int nrows, int nseg, int Kp,
                int k1, int fw, const float* __restrict__ rowthr, int* __restrict__ cidx, int4* __restrict__ meta,
                int* __restrict__ big, int* __restrict__ nbig) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * RW_WARPS + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int segn = (lane < nseg) ? cand_n[(int64_t)row * nseg + lane] : 0;
  int inc = segn;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  const int t = __shfl_sync(0xffffffffu, inc, 31);
  if (t > RW_MAXT) {  // the block kernel takes the row
    if (lane == 0) {
      meta[row] = make_int4(-1, 0, 0, 0);
      big[atomicAdd(nbig, 1)] = row;
    }
    return;
  }
  const float rthr = rowthr ? rowthr[row] : __int_as_float(0x7f800000);
  const int segoff = inc - segn;
  if (t <= 32)
    cands_row<1>(cand, row, nseg, Kp, k1, fw, t, segoff, segn, rthr, cidx, meta, lane);
  else if (t <= 64)
    cands_row<2>(cand, row, nseg, Kp, k1, fw, t, segoff, segn, rthr, cidx, meta, lane);
  else if (t <= 128)
    cands_row<4>(cand, row, nseg, Kp, k1, fw, t, segoff, segn, rthr, cidx, meta, lane);
  else if (t <= 256)
    cands_row<8>(cand, row, nseg, Kp, k1, fw, t, segoff, segn, rthr, cidx, meta, lane);
  else
    cands_row<16>(cand, row, nseg, Kp, k1, fw, t, segoff, segn, rthr, cidx, meta, lane);
}

// Stage 2, one thread per (row, candidate slot): the exact value of the
// candidate in the reference's arithmetic. The slots of all rows are one
// dense range, so every lane of the FP64 pipe has a pair to compute. For
// the correlation metric Xfit / Xref are the centred vectors (k_vec_center).
__global__ void __launch_bounds__(256)
k_recheck_exact(const double* __restrict__ Xfit, const double* __restrict__ Xref, const double* __restrict__ sfv,
                const double* __restrict__ srv, int nrows, int dim, int corr, int fw, const int* __restrict__ cidx,
                const int4* __restrict__ meta, double* __restrict__ ev) {
  const int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= (int64_t)nrows * fw) return;
  const int row = (int)(slot / fw), c = (int)(slot % fw);
  if (c >= meta[row].x) return;
  const int j = cidx[slot];
  const double* a = Xfit + (int64_t)row * dim;
  const double* b = Xref + (int64_t)j * dim;
  ev[slot] = corr ? exact_corr_centred(a, sfv[row], b, srv[j], dim) : exact_euclid(a, b, dim);
}

// Stage 3, one warp per row: the k+1 best rechecked candidates by (value,
// index). The row is done when the next candidate's bound lies above the
// (k+1)-th exact value and that value lies below tau, or when every
// candidate was rechecked (then dk < tau is required, else the row is
// flagged); otherwise it goes to the block kernel, which rechecks all its
// candidates.
__global__ void __launch_bounds__(RW_WARPS * 32)
k_recheck_finish(int nrows, int k, int fw, const int* __restrict__ cidx, const int4* __restrict__ meta,
                 const double* __restrict__ ev, double* __restrict__ out_d, int* __restrict__ out_i,
                 int* __restrict__ flagged, int* __restrict__ nflag, int* __restrict__ big, int* __restrict__ nbig) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * RW_WARPS + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int4 m = meta[row];
  const int first = m.x, total = m.y;
  if (first < 0) return;
  const float tau = __int_as_float(m.z), nxt = __int_as_float(m.w);
  const int k1 = k + 1;
  uint64_t v[4];
  int x[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = i * 32 + lane;
    v[i] = (e < first) ? (uint64_t)__double_as_longlong(ev[(int64_t)row * fw + e]) : 0x7ff0000000000000ull;
    x[i] = (e < first) ? cidx[(int64_t)row * fw + e] : 0x7fffffff;
  }
  wsort_pair<4>(v, x, lane);
  const uint64_t dkb = lane_elem<4>(v, k1 - 1);
  const double dk = __longlong_as_double((long long)dkb);
  if (first < total && !(dk < (double)nxt && dk < (double)tau)) {
    if (lane == 0) big[atomicAdd(nbig, 1)] = row;
    return;
  }
  // strict: a pair left out of the list has a lower bound >= tau, so only
  // dk < tau proves that no left-out pair ties with or beats the k+1-th
  if (lane == 0 && first == total && !(dk < (double)tau)) flagged[atomicAdd(nflag, 1)] = row;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int e = i * 32 + lane;
    if (e >= 1 && e <= k) {
      const bool have = e < first;
      out_d[(int64_t)row * k + e - 1] = have ? sqrt(__longlong_as_double((long long)v[i]))
                                             : __longlong_as_double(0x7ff0000000000000ll);
      out_i[(int64_t)row * k + e - 1] = have ? x[i] : 0x7fffffff;
    }
  }
}

static size_t data_recheck_smem(int dim, int Kp, int nseg, int k, int mode) {
  int k1 = k + 1;
  size_t merge = (mode == 0) ? (size_t)next_pow2(std::max(nseg * Kp, 1)) : 0;
  int CH = (mode == 0) ? next_pow2(std::max(Kp, 1)) : 1024;
  int BP2 = next_pow2(k1 + CH);
  size_t tail = (size_t)(mode == 0 ? Kp : 0) * 8 + (size_t)BP2 * (8 + 4);
  return sizeof(double) * dim + std::max(merge * 8, tail) + 64;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
int knn_data_run(mds_ctx* ctx, const double* dref, int nref, const double* dfit, int nfit, int dim, int k,
                 bool corr, bool full, unsigned prec, bool noskip, double* dout_d, int* dout_i) {
  cudaStream_t s = ctx->stream;
  mds_knn_stats& st = ctx->stats;
  const bool same = (dfit == nullptr);
  if (same) {
    dfit = dref;
    nfit = nref;
  }
  const int Dp = mds_round_up(dim, DT_KC);
  DevBuf Xr(ctx), Nrm(ctx), Mr(ctx), Sr(ctx), Xf(ctx), Nf(ctx), Mf(ctx), Sf(ctx), flagged(ctx), nflag(ctx);
  MDS_TRY(Xr.alloc(ctx, sizeof(float) * (size_t)nref * Dp));
  MDS_TRY(Nrm.alloc(ctx, sizeof(float) * nref));
  MDS_TRY(Mr.alloc(ctx, sizeof(double) * nref));
  MDS_TRY(Sr.alloc(ctx, sizeof(double) * nref));
  st.launches = 0;
  st.launches++;
  k_vec_prep<<<(nref + 127) / 128, 128, 0, s>>>(dref, nref, dim, Dp, corr, Xr.as<float>(), Nrm.as<float>(),
                                                Mr.as<double>(), Sr.as<double>());
  MDS_CUDA(ctx, cudaGetLastError());
  const float* xf = Xr.as<float>();
  const float* nfp = Nrm.as<float>();
  const double* mf = Mr.as<double>();
  const double* sf = Sr.as<double>();
  if (!same) {
    MDS_TRY(Xf.alloc(ctx, sizeof(float) * (size_t)nfit * Dp));
    MDS_TRY(Nf.alloc(ctx, sizeof(float) * nfit));
    MDS_TRY(Mf.alloc(ctx, sizeof(double) * nfit));
    MDS_TRY(Sf.alloc(ctx, sizeof(double) * nfit));
    st.launches++;
    k_vec_prep<<<(nfit + 127) / 128, 128, 0, s>>>(dfit, nfit, dim, Dp, corr, Xf.as<float>(), Nf.as<float>(),
                                                  Mf.as<double>(), Sf.as<double>());
    MDS_CUDA(ctx, cudaGetLastError());
    xf = Xf.as<float>();
    nfp = Nf.as<float>();
    mf = Mf.as<double>();
    sf = Sf.as<double>();
  }
  MDS_TRY(flagged.alloc(ctx, sizeof(int) * (size_t)std::max(nfit, 1)));
  MDS_TRY(nflag.alloc(ctx, sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(nflag.p, 0, sizeof(int), s));
  DevBuf big(ctx), nbig(ctx), cidx(ctx), meta(ctx), evals(ctx), Cr(ctx), Cf(ctx);
  auto recheck = [&](int nrows, const int* rowlist, int mode, const uint64_t* cand, const int* cand_n, int nseg,
                     int Kp, const float* rowthr) -> int {
    size_t smem = data_recheck_smem(dim, Kp, nseg, k, mode);
    if (smem > 227 * 1024) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "knn_data recheck: dim/k too large");
    if (mode == 0 && !rowlist && nrows > 0 && k + 1 <= RW_MAXK1) {
      // three stages (candidates, dense exact values, finish); the rows they
      // cannot finish go to the block kernel
      const int fw = k + 3;
      MDS_TRY(big.alloc(ctx, sizeof(int) * (size_t)nrows));
      MDS_TRY(nbig.alloc(ctx, sizeof(int)));
      MDS_TRY(cidx.alloc(ctx, sizeof(int) * (size_t)nrows * fw));
      MDS_TRY(meta.alloc(ctx, sizeof(int4) * (size_t)nrows));
      MDS_TRY(evals.alloc(ctx, sizeof(double) * (size_t)nrows * fw));
      MDS_CUDA(ctx, cudaMemsetAsync(nbig.p, 0, sizeof(int), s));
      const double* ea = dfit;
      const double* eb = dref;
      if (corr) {
        // centred copies of both sets (one for a set against itself)
        auto center = [&](const double* X, int n, const double* mean, DevBuf& out) -> int {
          const int64_t total = (int64_t)n * dim;
          MDS_TRY(out.alloc(ctx, sizeof(double) * (size_t)total));
          const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 8);
          st.launches++;
          k_vec_center<<<grid, 256, 0, s>>>(X, total, dim, mean, out.as<double>());
          MDS_CUDA(ctx, cudaGetLastError());
          return MDS_OK;
        };
        MDS_TRY(center(dref, nref, Mr.as<double>(), Cr));
        eb = ea = Cr.as<double>();
        if (!same) {
          MDS_TRY(center(dfit, nfit, mf, Cf));
          ea = Cf.as<double>();
        }
      }
      const int wb = (nrows + RW_WARPS - 1) / RW_WARPS;
      st.launches += 3;
      k_recheck_cands<<<wb, RW_WARPS * 32, 0, s>>>(cand, cand_n, nrows, nseg, Kp, k + 1, fw, rowthr, cidx.as<int>(),
                                                   meta.as<int4>(), big.as<int>(), nbig.as<int>());
      const int64_t slots = (int64_t)nrows * fw;
      k_recheck_exact<<<(int)((slots + 255) / 256), 256, 0, s>>>(ea, eb, sf, Sr.as<double>(), nrows, dim, corr, fw,
                                                                 cidx.as<int>(), meta.as<int4>(), evals.as<double>());
      k_recheck_finish<<<wb, RW_WARPS * 32, 0, s>>>(nrows, k, fw, cidx.as<int>(), meta.as<int4>(),
                                                    evals.as<double>(), dout_d, dout_i, flagged.as<int>(),
                                                    nflag.as<int>(), big.as<int>(), nbig.as<int>());
      MDS_CUDA(ctx, cudaGetLastError());
      int hbig = 0;
      MDS_CUDA(ctx, cudaMemcpyAsync(&hbig, nbig.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      st.recheck_pairs = slots;
      if (hbig == 0) return MDS_OK;
      rowlist = big.as<int>();
      nrows = hbig;
    }
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_data_recheck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    st.launches++;
    if (nrows > 0)
      k_data_recheck<<<nrows, DR_THREADS, smem, s>>>(dfit, dref, mf, sf, Mr.as<double>(), Sr.as<double>(), nfp,
                                                     nrows, rowlist, nref, dim, corr, mode, cand, cand_n, nseg, Kp,
                                                     k, rowthr, dout_d, dout_i, flagged.as<int>(), nflag.as<int>(),
                                                     rowlist == big.p ? 1 : 0);
    MDS_CUDA(ctx, cudaGetLastError());
    return MDS_OK;
  };
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  if (full) {
    MDS_TRY(recheck(nfit, nullptr, 2, nullptr, nullptr, 1, 1, nullptr));
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    st.recheck_ms = ms;
    return MDS_OK;
  }
  // K': the FP32 screen keeps a row's pool (K' + one tile) in shared memory,
  // which holds at most DT_MAX_KP; the tensor-core screen keeps its lists in
  // global memory and takes up to tcv_max_kprime()
  const int kp_want = mds_round_up(std::max(k + 1 + 32, (k + 1) * 3 / 2), 32);
  const bool tc = prec == MDS_PREC_BF16X3 && Dp <= tcv_max_dp() && kp_want <= tcv_max_kprime();
  int Kp = tc ? kp_want : std::min(kp_want, DT_MAX_KP);
  if (Kp < k + 1 + 16) {
    // k too large for a screen to pay off: every row is rechecked exactly
    st.kprime = 0;
    st.passes = 1;
    MDS_TRY(recheck(nfit, nullptr, 1, nullptr, nullptr, 1, 1, nullptr));
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    st.recheck_ms = ms;
    return MDS_OK;
  }
  const int nrt = (nfit + DT_TM - 1) / DT_TM, nct = (nref + DT_TN - 1) / DT_TN;
  int nseg = 1;
  {
    double besteff = 0;
    for (int sg = 1; sg <= 8 && sg <= nct; ++sg) {
      double w = (double)nrt * sg / ctx->num_sms, eff = w / std::ceil(w);
      if (eff > besteff + 0.02) {
        besteff = eff;
        nseg = sg;
      }
      if (eff >= 0.95) break;
    }
  }
  const float guard = MDS_GUARD_FP32;
  if (tc) nseg = tcv_choose_nseg(ctx, nfit, nref);
  DevBuf cand(ctx), cand_n(ctx), rows(ctx), rthr(ctx);
  MDS_TRY(cand.alloc(ctx, sizeof(uint64_t) * (size_t)nfit * nseg * Kp));
  MDS_TRY(cand_n.alloc(ctx, sizeof(int) * (size_t)nfit * nseg));
  size_t smem = screen_dot_smem(Kp);
  st.screen_launches = 1;
  if (tc) {
    MDS_TRY(rthr.alloc(ctx, sizeof(float) * (size_t)nfit));
    long long tiles = 0;
    MDS_TRY(launch_screen_tcv(ctx, xf, nfp, nfit, Xr.as<float>(), Nrm.as<float>(), nref, Dp, corr, Kp, k, nseg, same,
                              !noskip, cand.as<uint64_t>(), cand_n.as<int>(), rthr.as<float>(), &tiles));
    st.screen_pairs = tiles * 256LL * 128LL;
  } else {
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_screen_dot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    st.launches++;
    k_screen_dot<<<nrt * nseg, DT_THREADS, smem, s>>>(xf, Xr.as<float>(), nfp, Nrm.as<float>(), nfit, nullptr,
                                                       nref, Dp, corr, guard, Kp, nseg, cand.as<uint64_t>(),
                                                       cand_n.as<int>());
    MDS_CUDA(ctx, cudaGetLastError());
  }
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  MDS_TRY(recheck(nfit, nullptr, 0, cand.as<uint64_t>(), cand_n.as<int>(), nseg, Kp, tc ? rthr.as<float>() : nullptr));
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
  int hflag = 0;
  MDS_CUDA(ctx, cudaMemcpyAsync(&hflag, nflag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, ctx->ev[1], ctx->ev[2]);
  cudaEventElapsedTime(&b, ctx->ev[2], ctx->ev[3]);
  st.screen_ms = a;
  st.recheck_ms = b;
  st.kprime = Kp;
  st.rows_flagged = hflag;
  st.passes = 1;
  while (hflag > 0) {
    std::vector<int> hrows(hflag);
    MDS_CUDA(ctx, cudaMemcpyAsync(hrows.data(), flagged.p, sizeof(int) * hflag, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    std::sort(hrows.begin(), hrows.end());
    MDS_TRY(rows.alloc(ctx, sizeof(int) * hflag));
    MDS_CUDA(ctx, cudaMemcpyAsync(rows.p, hrows.data(), sizeof(int) * hflag, cudaMemcpyHostToDevice, s));
    MDS_CUDA(ctx, cudaMemsetAsync(nflag.p, 0, sizeof(int), s));
    st.passes++;
    const int wider = std::min(Kp * 4, DT_MAX_KP);
    if (wider <= Kp || wider >= nref || st.passes > 3) {
      MDS_TRY(recheck(hflag, rows.as<int>(), 1, nullptr, nullptr, 1, 1, nullptr));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      break;
    }
    Kp = wider;
    MDS_TRY(cand.alloc(ctx, sizeof(uint64_t) * (size_t)hflag * Kp));
    MDS_TRY(cand_n.alloc(ctx, sizeof(int) * (size_t)hflag));
    smem = screen_dot_smem(Kp);
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_screen_dot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    st.launches++;
    k_screen_dot<<<(hflag + DT_TM - 1) / DT_TM, DT_THREADS, smem, s>>>(xf, Xr.as<float>(), nfp, Nrm.as<float>(),
                                                                       hflag, rows.as<int>(), nref, Dp, corr, guard,
                                                                       Kp, 1, cand.as<uint64_t>(), cand_n.as<int>());
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_TRY(recheck(hflag, rows.as<int>(), 0, cand.as<uint64_t>(), cand_n.as<int>(), 1, Kp, nullptr));
    MDS_CUDA(ctx, cudaMemcpyAsync(&hflag, nflag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  return MDS_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant (mds_knn_data_noalloc). Some callers cannot obtain
// device memory at the point of the call: a plugin running inside another
// framework whose caching allocator has reserved the device memory in full
// (a cudaMalloc there fails, or takes memory the host framework counts on),
// or an embedding that forbids the library its own allocations. This entry
// point takes device inputs and outputs and keeps every scratch buffer in
// one file-scope device array of fixed size, so it never calls cudaMalloc
// or cudaFree. Every GPU that loads this library holds the array until the
// process exits.
// ---------------------------------------------------------------------------
#define MDS_NOALLOC_SCRATCH_BYTES (32u << 20)  // 32 MiB
#define MDS_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_knn_data_scratch[MDS_NOALLOC_SCRATCH_BYTES];

// Device address of the array. In host code g_knn_data_scratch names a
// host-side stand-in, so the address is taken with cudaGetSymbolAddress,
// once per device (std::call_once: safe from several host threads), with
// that device current. The caller's current device is left as it was.
static void* noalloc_scratch(int dev) {
  static std::once_flag once[MDS_NOALLOC_MAX_DEVICES];
  static void* addr[MDS_NOALLOC_MAX_DEVICES];
  if (dev < 0 || dev >= MDS_NOALLOC_MAX_DEVICES) return nullptr;
  std::call_once(once[dev], [dev] {
    int prev = -1;
    const bool had = cudaGetDevice(&prev) == cudaSuccess;
    void* p = nullptr;
    if (cudaSetDevice(dev) == cudaSuccess && cudaGetSymbolAddress(&p, g_knn_data_scratch) == cudaSuccess)
      addr[dev] = p;
    else
      cudaGetLastError();
    if (had) cudaSetDevice(prev);
  });
  return addr[dev];
}

// Makes ctx's device current for the call and puts the caller's back on
// every return path.
struct NoallocDeviceScope {
  int prev = -1;
  bool had = false;
  explicit NoallocDeviceScope(int dev) {
    had = cudaGetDevice(&prev) == cudaSuccess;
    cudaSetDevice(dev);
  }
  ~NoallocDeviceScope() {
    if (had) cudaSetDevice(prev);
  }
};

extern "C" int mds_knn_data_noalloc(mds_ctx* ctx, const double* ref, int n_ref, const double* fit, int n_fit,
                                    int dim, int k, unsigned flags, double* out_d, int32_t* out_i, int* k_used) {
  if (!ctx) return MDS_ERR_ARG;
  ctx->stats = mds_knn_stats{};
  if (!ref || !out_d || !out_i) return mds_fail(ctx, MDS_ERR_ARG, "null array argument");
  if (n_ref < 1 || dim < 1 || n_fit < 0)
    return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes: n_ref=%d n_fit=%d dim=%d", n_ref, n_fit, dim);
  if (flags & ~(MDS_CORRELATION | MDS_DEVICE_IO))
    return mds_fail(ctx, MDS_ERR_ARG, "mds_knn_data_noalloc accepts only MDS_CORRELATION (inputs are device pointers)");
  const bool corr = (flags & MDS_CORRELATION) != 0;
  const bool same = (fit == nullptr);
  if (same) n_fit = n_ref;
  if (k < 0) return mds_fail(ctx, MDS_ERR_ARG, "k must be >= 0");
  if (n_ref - 1 < k) k = n_ref - 1;  // knn_data.cpp:186-188
  if (k_used) *k_used = k;
  if (n_fit == 0 || k == 0) return MDS_OK;
  const int Dp = mds_round_up(dim, DT_KC);
  // K' as mds_knn_data's FP32 screen chooses it, within the screen's shared
  // memory pools; when that leaves fewer than 16 spare candidates the screen
  // does not pay off and every row is rechecked exactly (as mds_knn_data)
  const int Kp = std::min(mds_round_up(std::max(k + 1 + 32, (k + 1) * 3 / 2), 32), DT_MAX_KP);
  const bool exact_rows = Kp < k + 1 + 16;
  // scratch layout, 256-byte aligned pieces
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t need = 0;
  const size_t o_xr = need;  need += up(sizeof(float) * (size_t)n_ref * Dp);
  const size_t o_nr = need;  need += up(sizeof(float) * (size_t)n_ref);
  const size_t o_mr = need;  need += up(sizeof(double) * (size_t)n_ref);
  const size_t o_sr = need;  need += up(sizeof(double) * (size_t)n_ref);
  size_t o_xf = 0, o_nf = 0, o_mf = 0, o_sf = 0;
  if (!same) {
    o_xf = need;  need += up(sizeof(float) * (size_t)n_fit * Dp);
    o_nf = need;  need += up(sizeof(float) * (size_t)n_fit);
    o_mf = need;  need += up(sizeof(double) * (size_t)n_fit);
    o_sf = need;  need += up(sizeof(double) * (size_t)n_fit);
  }
  size_t o_cand = 0, o_cn = 0;
  if (!exact_rows) {
    o_cand = need;  need += up(sizeof(uint64_t) * (size_t)n_fit * Kp);
    o_cn = need;    need += up(sizeof(int) * (size_t)n_fit);
  }
  const size_t o_fl = need;    need += up(sizeof(int) * (size_t)n_fit);
  const size_t o_nfl = need;   need += up(sizeof(int));
  if (need > MDS_NOALLOC_SCRATCH_BYTES)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED,
                    "mds_knn_data_noalloc: this problem needs %zu bytes of scratch, more than the fixed %u bytes "
                    "(use mds_knn_data)", need, (unsigned)MDS_NOALLOC_SCRATCH_BYTES);
  unsigned char* base = static_cast<unsigned char*>(noalloc_scratch(ctx->device));
  if (!base) return mds_fail(ctx, MDS_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
  NoallocDeviceScope scope(ctx->device);
  cudaStream_t s = ctx->stream;
  float* xr = reinterpret_cast<float*>(base + o_xr);
  float* nr = reinterpret_cast<float*>(base + o_nr);
  double* mr = reinterpret_cast<double*>(base + o_mr);
  double* sr = reinterpret_cast<double*>(base + o_sr);
  const float* nf = nr;
  const double* mf = mr;
  const double* sf = sr;
  const float* xf = xr;
  k_vec_prep<<<(n_ref + 127) / 128, 128, 0, s>>>(ref, n_ref, dim, Dp, corr, xr, nr, mr, sr);
  ctx->stats.launches++;
  if (!same) {
    float* xf2 = reinterpret_cast<float*>(base + o_xf);
    float* nf2 = reinterpret_cast<float*>(base + o_nf);
    double* mf2 = reinterpret_cast<double*>(base + o_mf);
    double* sf2 = reinterpret_cast<double*>(base + o_sf);
    k_vec_prep<<<(n_fit + 127) / 128, 128, 0, s>>>(fit, n_fit, dim, Dp, corr, xf2, nf2, mf2, sf2);
    ctx->stats.launches++;
    xf = xf2; nf = nf2; mf = mf2; sf = sf2;
  }
  MDS_CUDA(ctx, cudaGetLastError());
  const double* dfit = same ? ref : fit;
  int* flagged = reinterpret_cast<int*>(base + o_fl);
  int* nflag = reinterpret_cast<int*>(base + o_nfl);
  if (exact_rows) {
    size_t rsm = data_recheck_smem(dim, 1, 1, k, 1);
    if (rsm > 227 * 1024) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "dim/k too large");
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_data_recheck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
    k_data_recheck<<<n_fit, DR_THREADS, rsm, s>>>(dfit, ref, mf, sf, mr, sr, nf, n_fit, nullptr, n_ref, dim, corr, 1,
                                                  nullptr, nullptr, 1, 1, k, nullptr, out_d, out_i, nullptr, nullptr, 0);
    ctx->stats.launches++;
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->stats.passes = 1;
    return MDS_OK;
  }
  uint64_t* cand = reinterpret_cast<uint64_t*>(base + o_cand);
  int* cand_n = reinterpret_cast<int*>(base + o_cn);
  // the array keeps the previous call's contents: the flag counter restarts at zero
  MDS_CUDA(ctx, cudaMemsetAsync(nflag, 0, sizeof(int), s));
  const size_t ssm = screen_dot_smem(Kp);
  MDS_CUDA(ctx, cudaFuncSetAttribute(k_screen_dot, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
  const int nrt = (n_fit + DT_TM - 1) / DT_TM;
  k_screen_dot<<<nrt, DT_THREADS, ssm, s>>>(xf, xr, nf, nr, n_fit, nullptr, n_ref, Dp, corr, MDS_GUARD_FP32, Kp, 1,
                                            cand, cand_n);
  ctx->stats.launches++;
  MDS_CUDA(ctx, cudaGetLastError());
  size_t rsm = data_recheck_smem(dim, Kp, 1, k, 0);
  if (rsm > 227 * 1024) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "dim/k too large");
  MDS_CUDA(ctx, cudaFuncSetAttribute(k_data_recheck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
  k_data_recheck<<<n_fit, DR_THREADS, rsm, s>>>(dfit, ref, mf, sf, mr, sr, nf, n_fit, nullptr, n_ref, dim, corr, 0,
                                                cand, cand_n, 1, Kp, k, nullptr, out_d, out_i, flagged, nflag, 0);
  ctx->stats.launches++;
  MDS_CUDA(ctx, cudaGetLastError());
  int hflag = 0;
  MDS_CUDA(ctx, cudaMemcpyAsync(&hflag, nflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  ctx->stats.kprime = Kp;
  ctx->stats.rows_flagged = hflag;
  ctx->stats.passes = 1;
  if (hflag > 0) {
    // rows whose guard check failed: every reference vector is rechecked
    // exactly; the flagged list is only read here (exact rows flag nothing)
    rsm = data_recheck_smem(dim, 1, 1, k, 1);
    if (rsm > 227 * 1024) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "dim/k too large");
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_data_recheck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
    k_data_recheck<<<hflag, DR_THREADS, rsm, s>>>(dfit, ref, mf, sf, mr, sr, nf, hflag, flagged, n_ref, dim, corr, 1,
                                                  nullptr, nullptr, 1, 1, k, nullptr, out_d, out_i, nullptr, nullptr, 0);
    ctx->stats.launches++;
    ctx->stats.passes = 2;
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  return MDS_OK;
}
