// vec_order.cu -- locality order and tile bounds for the tensor-core vector
// screen of knn_data (knn_data_tc.cu).
//
// knn_data.cpp:195-250 compares every fit vector with every reference vector.
// Its inputs (sin/cos of dihedral angles, or any feature vectors) need not be
// stored in any useful order, so the screen's column tiles are, for a given
// row, a random sample of the set: its threshold tightens slowly, and no tile
// can be left out. This file reorders both sets so that tiles are compact,
// and bounds, for every (row pair tile, column tile), the distance of any of
// its pairs from below:
//
//  1. k-means with VO_CENT centroids (Lloyd iterations, the centroids seeded
//     with evenly spaced vectors), then a stable sort by (centroid, distance
//     to it quantised to 12 bits): a tile holds vectors of one cluster at
//     about one distance from its centroid. The order changes which pairs the
//     screen computes, never the result: the recheck works on the original
//     indices and recomputes every candidate exactly.
//  2. Per column tile, its centre c (FP32 mean of its vectors) and radius
//     rho = max |y - c| (accumulated in FP64 against the FP32 centre, rounded
//     up).
//  3. Per row pair tile I and column tile T, dlo, a lower bound of the
//     distance of every pair (x in I, y in T) by the triangle inequality: when
//     dlo > 0 and dlo^2 is at least every row's current threshold, none of
//     the tile's pairs can enter any row's list, and the screen skips it.
//     First coarsely from I's own centre and radius, |c_I - c_T| - rho_I -
//     rho_T; then, where that cannot prove a skip against the rows' threshold
//     seeds, min over the rows x of I of |x - c_T| - rho_T (FP32, with margins
//     for its rounding and the inputs' rounding to FP32). Also the start tile
//     of each (row pair tile, column segment) visit: the one with the
//     smallest dlo.
#include <algorithm>

#include "knn_common.cuh"

#define VO_CENT 16
#define VO_ITERS 6
#define VO_MAXDP 128
#define VO_QBITS 12

// centroid c := vector (2c + 1) n / (2 VO_CENT)
__global__ void k_vo_seed(const float* __restrict__ X, int n, int Dp, float* __restrict__ cent) {
  const int c = blockIdx.x;
  const int64_t v = (int64_t)(2 * c + 1) * n / (2 * VO_CENT);
  for (int d = threadIdx.x; d < Dp; d += blockDim.x) cent[c * Dp + d] = X[v * Dp + d];
}

// Nearest centroid of every stride-th vector. sums/counts (zeroed by the
// caller): the FP64 sums and counts of each centroid's vectors, for the next
// centroids.
// keys/vals: (centroid << 12 | distance quantised against *dmax) and the
// vector's index, for the sort; dist/dmax: the distance to the nearest
// centroid and (float bits) the largest one, for that quantisation.
__global__ void __launch_bounds__(256) k_vo_assign(const float* __restrict__ X, int n, int Dp, int stride,
                                                   const float* __restrict__ cent, double* __restrict__ sums,
                                                   int* __restrict__ counts, float* __restrict__ dist,
                                                   unsigned* __restrict__ dmax, int* __restrict__ label) {
  __shared__ float cs[VO_CENT * VO_MAXDP];
  __shared__ double ss[VO_CENT * VO_MAXDP];
  __shared__ int sc[VO_CENT];
  for (int e = threadIdx.x; e < VO_CENT * Dp; e += blockDim.x) {
    cs[e] = cent[e];
    if (sums) ss[e] = 0.0;
  }
  if (threadIdx.x < VO_CENT) sc[threadIdx.x] = 0;
  __syncthreads();
  const int64_t v = (int64_t)(blockIdx.x * blockDim.x + threadIdx.x) * stride;
  float best = __int_as_float(0x7f800000);
  int bl = 0;
  if (v < n) {
    const float4* x4 = reinterpret_cast<const float4*>(X + (int64_t)v * Dp);
    float acc[VO_CENT];
#pragma unroll
    for (int c = 0; c < VO_CENT; ++c) acc[c] = 0.0f;
    for (int q = 0; q < Dp / 4; ++q) {
      const float4 xv = x4[q];
#pragma unroll
      for (int c = 0; c < VO_CENT; ++c) {
        const float* cc = cs + c * Dp + 4 * q;
        float e = xv.x - cc[0];
        acc[c] = fmaf(e, e, acc[c]);
        e = xv.y - cc[1];
        acc[c] = fmaf(e, e, acc[c]);
        e = xv.z - cc[2];
        acc[c] = fmaf(e, e, acc[c]);
        e = xv.w - cc[3];
        acc[c] = fmaf(e, e, acc[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < VO_CENT; ++c)
      if (acc[c] < best) {
        best = acc[c];
        bl = c;
      }
    if (sums) {
      for (int d = 0; d < Dp; ++d) atomicAdd(&ss[bl * Dp + d], (double)X[(int64_t)v * Dp + d]);
      atomicAdd(&sc[bl], 1);
    }
    if (dist) {
      const float dv = sqrtf(best);
      dist[v] = dv;
      label[v] = bl;
      atomicMax(dmax, __float_as_uint(dv));
    }
  }
  if (sums) {
    __syncthreads();
    for (int e = threadIdx.x; e < VO_CENT * Dp; e += blockDim.x)
      if (ss[e] != 0.0) atomicAdd(&sums[e], ss[e]);
    if (threadIdx.x < VO_CENT && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
  }
}

// New centroids from the sums (a centroid without vectors stays); the sums
// and counts are cleared for the next iteration.
__global__ void k_vo_update(float* __restrict__ cent, double* __restrict__ sums, int* __restrict__ counts, int Dp) {
  const int c = blockIdx.x;
  const int cnt = counts[c];
  for (int d = threadIdx.x; d < Dp; d += blockDim.x) {
    if (cnt > 0) cent[c * Dp + d] = (float)(sums[c * Dp + d] / cnt);
    sums[c * Dp + d] = 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) counts[c] = 0;
}

__global__ void k_vo_keys(const int* __restrict__ label, const float* __restrict__ dist,
                          const unsigned* __restrict__ dmax, int n, unsigned long long* __restrict__ keys,
                          int64_t* __restrict__ vals) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const float dm = __uint_as_float(*dmax);
  const float qs = (dm > 0.0f) ? (float)(1 << VO_QBITS) / dm : 0.0f;
  const int q = min((1 << VO_QBITS) - 1, (int)(dist[v] * qs));
  keys[v] = ((unsigned long long)label[v] << VO_QBITS) | (unsigned)q;
  vals[v] = v;
}

__global__ void k_vo_perm(const int64_t* __restrict__ vals, int n, int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[i] = (int)vals[i];
}

// Column tile T = sorted vectors [T * tile, T * tile + tile): FP32 centre and
// radius (rounded up). Block: `tile` threads.
__global__ void k_vo_tile_geom(const float* __restrict__ X, const int* __restrict__ perm, int n, int Dp, int tile,
                               float* __restrict__ center, float* __restrict__ rad) {
  __shared__ float cf[VO_MAXDP];
  __shared__ float red[32];
  const int T = blockIdx.x, t = threadIdx.x;
  const int j0 = T * tile, m = min(tile, n - j0);
  for (int d = t; d < Dp; d += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += (double)X[(int64_t)perm[j0 + j] * Dp + d];
    cf[d] = (float)(s / m);
    center[(int64_t)T * Dp + d] = cf[d];
  }
  __syncthreads();
  float r = 0.0f;
  if (t < m) {
    const float* y = X + (int64_t)perm[j0 + t] * Dp;
    double s = 0.0;
    for (int d = 0; d < Dp; ++d) {
      const double e = (double)y[d] - (double)cf[d];
      s += e * e;
    }
    r = __double2float_ru(sqrt(s) * (1.0 + 1e-7));
  }
  for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, o));
  if ((t & 31) == 0) red[t >> 5] = r;
  __syncthreads();
  if (t == 0) {
    float mx = 0.0f;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) mx = fmaxf(mx, red[w]);
    rad[T] = mx;
  }
}

// Ascending bitonic sort of 128 values held 4 per lane (element 4 lane + i).
__device__ __forceinline__ void warp_sort128(float (&v)[4], int lane) {
#pragma unroll
  for (int k = 2; k <= 128; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 4) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int e = lane * 4 + i;
          const float o = __shfl_xor_sync(0xffffffffu, v[i], j >> 2);
          v[i] = (((e & j) == 0) == ((e & k) == 0)) ? fminf(v[i], o) : fmaxf(v[i], o);
        }
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int p = i ^ j;
          if (p > i) {
            const bool up = ((lane * 4 + i) & k) == 0;
            const float a = v[i], b = v[p];
            if ((a > b) == up) {
              v[i] = b;
              v[p] = a;
            }
          }
        }
      }
    }
  }
}

// Seeds the threshold of every sorted fit row: its k1-th smallest squared
// distance to the members of its start tile (the diagonal tile for a set
// against itself, else tdall[row pair tile]), raised by a margin for the
// FP32 arithmetic -- an upper bound of the row's k1-th smallest over the
// whole reference set, which holds those members. Block: one row pair tile,
// 8 warps taking its rows in turn (lane j: members j, j + 32, j + 64, j + 96).
// Rows whose start tile has fewer than k1 members keep +inf.
__global__ void __launch_bounds__(256) k_vo_seed_rows(const float* __restrict__ Xr, const int* __restrict__ permr,
                                                      int nref, const float* __restrict__ Xf,
                                                      const int* __restrict__ permf, int nfit, int Dp,
                                                      const int* __restrict__ tdall, int ncoltiles, int k1,
                                                      const float* __restrict__ nmax, float* __restrict__ rowthr,
                                                      const unsigned* __restrict__ devn) {
  extern __shared__ float sm[];  // members [128][Dp + 1], then rows [8][Dp]
  const int item = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int T = tdall ? tdall[item] : min((item * 256 + 128) / 128, ncoltiles - 1);
  const int j0 = T * 128, m = min(128, nref - j0);
  const int ld = Dp + 1;
  float* mem = sm;
  float* rowv = sm + 128 * ld + w * Dp;
  for (int e = threadIdx.x; e < 128 * Dp; e += blockDim.x) {
    const int j = e / Dp, d = e % Dp;
    mem[j * ld + d] = (j < m) ? Xr[(int64_t)permr[j0 + j] * Dp + d] : 0.0f;
  }
  __syncthreads();
  const float nm = __ldg(nmax);
  for (int r = w; r < 256; r += 8) {
    const int g = item * 256 + r;
    if (g >= nfit) break;
    const float* x = Xf + (int64_t)permf[g] * Dp;
    for (int d = lane; d < Dp; d += 32) rowv[d] = x[d];
    __syncwarp();
    float v[4];
    float xn = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int j = lane + 32 * i;
      const float* y = mem + j * ld;
      float s0 = 0.0f, s1 = 0.0f;
      for (int d = 0; d < Dp; d += 2) {
        const float e0 = rowv[d] - y[d], e1 = rowv[d + 1] - y[d + 1];
        s0 = fmaf(e0, e0, s0);
        s1 = fmaf(e1, e1, s1);
      }
      v[i] = (j < m) ? s0 + s1 : __int_as_float(0x7f800000);
    }
    for (int d = 0; d < Dp; ++d) xn = fmaf(rowv[d], rowv[d], xn);
    warp_sort128(v, lane);
    const int q = k1 - 1;
    const float vk = __shfl_sync(0xffffffffu, v[q & 3], q >> 2);
    // the FP32 sum of Dp squares errs by < (Dp + 2) 2^-24 of itself; the
    // inputs' rounding to FP32 moves d^2 by < 2.4e-7 (|x|^2 + |y|^2)
    // (correlation: the distance is a quarter of that within corr_margin)
    const float up = vk * (1.0f + 3e-5f) + 1e-6f * (xn + nm);
    if (lane == 0 && k1 <= m) rowthr[g] = devn ? 0.25f * up + corr_margin(devn, Dp) : up;
    __syncwarp();
  }
}

// Coarse bound of every (row pair tile I, column tile T): with c_I, rho_I the
// item's centre and radius (k_vo_tile_geom over 256-row tiles), every pair
// has |x - y| >= |c_I - c_T| - rho_I - rho_T. |x| <= |c_I| + rho_I bounds the
// rows' norms in the absolute margin. Grid (items, ceil(nct / 256)).
__global__ void __launch_bounds__(256) k_vo_coarse(const float* __restrict__ cenI, const float* __restrict__ radI,
                                                   const float* __restrict__ cenT, const float* __restrict__ radT,
                                                   int nct, int Dp, const float* __restrict__ nmax,
                                                   float* __restrict__ dlo) {
  __shared__ float ci[VO_MAXDP];
  const int item = blockIdx.x, T = blockIdx.y * blockDim.x + threadIdx.x;
  for (int d = threadIdx.x; d < Dp; d += blockDim.x) ci[d] = cenI[(int64_t)item * Dp + d];
  __syncthreads();
  if (T >= nct) return;
  float s0 = 0.0f, s1 = 0.0f, cn = 0.0f;
  const float* ct = cenT + (int64_t)T * Dp;
  for (int d = 0; d < Dp; d += 2) {
    const float e0 = ci[d] - ct[d], e1 = ci[d + 1] - ct[d + 1];
    s0 = fmaf(e0, e0, s0);
    s1 = fmaf(e1, e1, s1);
    cn = fmaf(ci[d], ci[d], fmaf(ci[d + 1], ci[d + 1], cn));
  }
  const float rI = __ldg(radI + item);
  const float nabs = 2e-6f * (sqrtf(__ldg(nmax)) + sqrtf(cn) + rI);
  dlo[(int64_t)item * nct + T] = sqrtf(s0 + s1) * (1.0f - 3e-5f) - rI - __ldg(radT + T) - nabs;
}

// Refines dlo[I][T] where the coarse bound cannot prove a skip: a tile is
// skipped when dlo > 0 and dlo^2 is at least the largest threshold of the
// item's rows, and those only fall from their seeds (rowthr on entry), so a
// coarse dlo with dlo^2 >= the largest seed already skips and is kept. The
// others (gathered 256 tiles at a time, computed 32 at a time; blockDim.x =
// 256 sorted rows, rows past n absent) get min over the rows x of |x - c_T|
// minus rho_T and the margins, the larger of the two bounds kept:
//   |x - c|^2 = |x|^2 + |c|^2 - 2 x.c in FP32 (one FMA per dimension): each
//   of the three terms errs by at most ~DP 2^-24 (|x|^2 + |c|^2), so
//   4e-7 DP (|x|^2 + |c|^2) taken off before the square root keeps it a
//   lower bound; |x32 - x| <= 2^-24 |x| for each input vector, which
//   2e-6 (|x|max + |y|max) covers with room.
template <int DP>
__global__ void __launch_bounds__(256) k_vo_refine(const float* __restrict__ X, const int* __restrict__ perm, int n,
                                                   const float* __restrict__ center, const float* __restrict__ rad,
                                                   int nct, const float* __restrict__ nmax,
                                                   const float* __restrict__ rowthr, float* __restrict__ dlo,
                                                   const unsigned* __restrict__ devn) {
  __shared__ __align__(16) float cen[32 * DP];
  __shared__ float cnr[32];
  __shared__ float wmin[8][33];
  __shared__ int list[256];
  __shared__ int s_cnt;
  const int item = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int g = item * 256 + t;
  const bool valid = g < n;
  float x[DP];
  if (valid) {
    const float4* x4 = reinterpret_cast<const float4*>(X + (int64_t)perm[g] * DP);
#pragma unroll
    for (int q = 0; q < DP / 4; ++q) {
      const float4 v = x4[q];
      x[4 * q] = v.x;
      x[4 * q + 1] = v.y;
      x[4 * q + 2] = v.z;
      x[4 * q + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int d = 0; d < DP; ++d) x[d] = 0.0f;
  }
  float xn0 = 0.0f, xn1 = 0.0f;
#pragma unroll
  for (int d = 0; d < DP; d += 2) {
    xn0 = fmaf(x[d], x[d], xn0);
    xn1 = fmaf(x[d + 1], x[d + 1], xn1);
  }
  const float xn = xn0 + xn1;
  // the rows' largest norm and largest seed (both non-negative: as unsigned bits)
  unsigned xm = __reduce_max_sync(0xffffffffu, __float_as_uint(xn));
  unsigned sm = __reduce_max_sync(0xffffffffu, valid ? __float_as_uint(fmaxf(__ldcg(rowthr + g), 0.0f)) : 0u);
  if (lane == 0) {
    wmin[w][31] = __uint_as_float(xm);
    wmin[w][32] = __uint_as_float(sm);
  }
  __syncthreads();
  float xmax = 0.0f, smax = 0.0f;
  for (int k = 0; k < 8; ++k) {
    xmax = fmaxf(xmax, wmin[k][31]);
    smax = fmaxf(smax, wmin[k][32]);
  }
  __syncthreads();
  const float nabs = 2e-6f * (sqrtf(__ldg(nmax)) + sqrtf(xmax));
  const float mrel = 4e-7f * DP;
  // the distance as a function of |x - y| (correlation: see k_vo_seed_rows)
  const float dsc = devn ? 0.25f : 1.0f;
  const float dmarg = devn ? corr_margin(devn, DP) : 0.0f;
  float* row = dlo + (int64_t)item * nct;
  for (int W0 = 0; W0 < nct; W0 += 256) {
    // the tiles of this window that the coarse bound cannot skip (the first
    // barrier: every thread has read the last window's count and list)
    __syncthreads();
    if (t == 0) s_cnt = 0;
    __syncthreads();
    {
      const int T = W0 + t;
      const float c = (T < nct) ? row[T] : 1.0f;
      const bool need = T < nct && !(c > 0.0f && c * c * dsc - dmarg >= smax);
      const unsigned b = __ballot_sync(0xffffffffu, need);
      int base = 0;
      if (lane == 0 && b) base = atomicAdd(&s_cnt, __popc(b));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (need) list[base + __popc(b & ((1u << lane) - 1u))] = T;
    }
    __syncthreads();
    const int nl = s_cnt;
    for (int L0 = 0; L0 < nl; L0 += 32) {
      const int nt = min(32, nl - L0);
      __syncthreads();
      for (int e = t; e < nt * DP; e += 256) cen[e] = center[(int64_t)list[L0 + e / DP] * DP + e % DP];
      __syncthreads();
      if (t < nt) {
        float c0 = 0.0f, c1 = 0.0f;
        for (int d = 0; d < DP; d += 2) {
          c0 = fmaf(cen[t * DP + d], cen[t * DP + d], c0);
          c1 = fmaf(cen[t * DP + d + 1], cen[t * DP + d + 1], c1);
        }
        cnr[t] = c0 + c1;
      }
      __syncthreads();
      for (int tt = 0; tt < nt; ++tt) {
        const float4* c4 = reinterpret_cast<const float4*>(cen + tt * DP);
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
        for (int q = 0; q < DP / 4; ++q) {
          const float4 c = c4[q];
          s0 = fmaf(x[4 * q], c.x, s0);
          s1 = fmaf(x[4 * q + 1], c.y, s1);
          s2 = fmaf(x[4 * q + 2], c.z, s2);
          s3 = fmaf(x[4 * q + 3], c.w, s3);
        }
        const float cn = cnr[tt];
        const float d2 = fmaxf((xn + cn) - 2.0f * ((s0 + s1) + (s2 + s3)) - mrel * (xn + cn), 0.0f);
        unsigned u = valid ? __float_as_uint(d2) : 0x7f800000u;
        u = __reduce_min_sync(0xffffffffu, u);
        if (lane == 0) wmin[w][tt] = __uint_as_float(u);
      }
      __syncthreads();
      if (w == 0 && lane < nt) {
        float m = wmin[0][lane];
#pragma unroll
        for (int k = 1; k < 8; ++k) m = fminf(m, wmin[k][lane]);
        const int T = list[L0 + lane];
        row[T] = fmaxf(row[T], sqrtf(m) * (1.0f - 1e-6f) - __ldg(rad + T) - nabs);
      }
    }
  }
}

// Start tile of each (row pair tile, segment) visit: the smallest dlo in the
// segment (lowest tile on ties). blockIdx.y == nseg: over all tiles (the
// pilot's start). One warp per block.
__global__ void k_vo_start(const float* __restrict__ dlo, int nct, int nseg, int* __restrict__ tdseg,
                           int* __restrict__ tdall, int only_all) {
  const int item = blockIdx.x, sg = only_all ? nseg : (int)blockIdx.y, lane = threadIdx.x;
  const int t0 = (sg == nseg) ? 0 : (int)((int64_t)nct * sg / nseg);
  const int t1 = (sg == nseg) ? nct : (int)((int64_t)nct * (sg + 1) / nseg);
  const float* row = dlo + (int64_t)item * nct;
  float bv = __int_as_float(0x7f800000);
  int bt = t0;
  for (int T = t0 + lane; T < t1; T += 32) {
    const float v = row[T];
    if (v < bv) {
      bv = v;
      bt = T;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const int ot = __shfl_xor_sync(0xffffffffu, bt, o);
    if (ov < bv || (ov == bv && ot < bt)) {
      bv = ov;
      bt = ot;
    }
  }
  if (lane == 0) {
    if (sg == nseg) {
      if (tdall) tdall[item] = bt;
    } else {
      tdseg[(int64_t)item * nseg + sg] = bt;
    }
  }
}

__global__ void k_vo_unsort(const float* __restrict__ src, const int* __restrict__ perm, int n,
                            float* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}

int vec_order_max_dp() { return VO_MAXDP; }

// perm[i] = original index of the i-th vector in locality order. cent
// ([VO_CENT][Dp]): fit == true computes the centroids (k-means from seeds),
// else they are given (a second set ordered by the first set's centroids).
int vec_order(mds_ctx* ctx, const float* X, int n, int Dp, float* cent, bool fit, int* perm) {
  if (Dp > VO_MAXDP || Dp % 4) return mds_fail(ctx, MDS_ERR_INTERNAL, "vec_order: padded dimension %d", Dp);
  cudaStream_t s = ctx->stream;
  DevBuf sums(ctx), counts(ctx), dist(ctx), label(ctx), dmax(ctx), k0(ctx), v0(ctx), k1(ctx), v1(ctx);
  MDS_TRY(dist.alloc(ctx, sizeof(float) * (size_t)n));
  MDS_TRY(label.alloc(ctx, sizeof(int) * (size_t)n));
  MDS_TRY(dmax.alloc(ctx, sizeof(unsigned)));
  MDS_CUDA(ctx, cudaMemsetAsync(dmax.p, 0, sizeof(unsigned), s));
  const int nb = (n + 255) / 256;
  if (fit) {
    MDS_TRY(sums.alloc(ctx, sizeof(double) * VO_CENT * Dp));
    MDS_TRY(counts.alloc(ctx, sizeof(int) * VO_CENT));
    MDS_CUDA(ctx, cudaMemsetAsync(sums.p, 0, sizeof(double) * VO_CENT * Dp, s));
    MDS_CUDA(ctx, cudaMemsetAsync(counts.p, 0, sizeof(int) * VO_CENT, s));
    k_vo_seed<<<VO_CENT, 128, 0, s>>>(X, n, Dp, cent);
    ctx->stats.launches++;
    // the iterations run on an evenly strided sample of about 16 k vectors
    const int stride = std::max(1, n / 16384);
    const int nbs = ((n + stride - 1) / stride + 255) / 256;
    for (int it = 0; it < VO_ITERS; ++it) {
      k_vo_assign<<<nbs, 256, 0, s>>>(X, n, Dp, stride, cent, sums.as<double>(), counts.as<int>(), nullptr,
                                      nullptr, nullptr);
      k_vo_update<<<VO_CENT, 128, 0, s>>>(cent, sums.as<double>(), counts.as<int>(), Dp);
      ctx->stats.launches += 2;
    }
  }
  k_vo_assign<<<nb, 256, 0, s>>>(X, n, Dp, 1, cent, nullptr, nullptr, dist.as<float>(), dmax.as<unsigned>(),
                                 label.as<int>());
  MDS_TRY(k0.alloc(ctx, sizeof(unsigned long long) * (size_t)n));
  MDS_TRY(v0.alloc(ctx, sizeof(int64_t) * (size_t)n));
  MDS_TRY(k1.alloc(ctx, sizeof(unsigned long long) * (size_t)n));
  MDS_TRY(v1.alloc(ctx, sizeof(int64_t) * (size_t)n));
  k_vo_keys<<<nb, 256, 0, s>>>(label.as<int>(), dist.as<float>(), dmax.as<unsigned>(), n,
                               k0.as<unsigned long long>(), v0.as<int64_t>());
  ctx->stats.launches += 2;
  MDS_CUDA(ctx, cudaGetLastError());
  int which = 0;
  MDS_TRY(radix_sort(ctx, k0.as<unsigned long long>(), v0.as<int64_t>(), k1.as<unsigned long long>(),
                     v1.as<int64_t>(), n, (1ull << (VO_QBITS + 4)) - 1, &which));
  k_vo_perm<<<nb, 256, 0, s>>>(which ? v1.as<int64_t>() : v0.as<int64_t>(), n, perm);
  ctx->stats.launches++;
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// Column tile geometry of the sorted reference set (tiles of `tile` = 128
// vectors), the row pair tiles' geometry (256 sorted fit rows), the coarse
// bounds dlo [nitems][nct], tdall [nitems] (the start over all tiles; null
// for a set against itself), the threshold seeds of the rows into rowthr
// (sorted order, +inf-like before), then the refinement of the bounds the
// coarse ones cannot skip by, and tdseg [nitems][nseg] (or null). nmax:
// device float, the reference set's largest squared norm. devn (or null):
// the correlation metric's largest | |z|^2 - 1 | (float bits).
int vec_tile_bounds(mds_ctx* ctx, const float* Xr, const int* permr, int nref, const float* Xf, const int* permf,
                    int nfit, int Dp, int tile, const float* nmax, float* dlo, int nseg, int* tdseg, int* tdall,
                    int k1, float* rowthr, const unsigned* devn) {
  cudaStream_t s = ctx->stream;
  const int nct = (nref + tile - 1) / tile, nitems = (nfit + 255) / 256;
  DevBuf center(ctx), rad(ctx), cenI(ctx), radI(ctx);
  MDS_TRY(center.alloc(ctx, sizeof(float) * (size_t)nct * Dp));
  MDS_TRY(rad.alloc(ctx, sizeof(float) * (size_t)nct));
  MDS_TRY(cenI.alloc(ctx, sizeof(float) * (size_t)nitems * Dp));
  MDS_TRY(radI.alloc(ctx, sizeof(float) * (size_t)nitems));
  k_vo_tile_geom<<<nct, tile, 0, s>>>(Xr, permr, nref, Dp, tile, center.as<float>(), rad.as<float>());
  k_vo_tile_geom<<<nitems, 256, 0, s>>>(Xf, permf, nfit, Dp, 256, cenI.as<float>(), radI.as<float>());
  k_vo_coarse<<<dim3(nitems, (nct + 255) / 256), 256, 0, s>>>(cenI.as<float>(), radI.as<float>(), center.as<float>(),
                                                               rad.as<float>(), nct, Dp, nmax, dlo);
  ctx->stats.launches += 3;
  if (tdall) {
    k_vo_start<<<dim3(nitems, 1), 32, 0, s>>>(dlo, nct, nseg, nullptr, tdall, 1);
    ctx->stats.launches++;
  }
  MDS_CUDA(ctx, cudaGetLastError());
  MDS_TRY(vec_seed_rows(ctx, Xr, permr, nref, Xf, permf, nfit, Dp, tdall, k1, nmax, rowthr, devn));
  switch (Dp) {
    case 32:
      k_vo_refine<32><<<nitems, 256, 0, s>>>(Xf, permf, nfit, center.as<float>(), rad.as<float>(), nct, nmax,
                                             rowthr, dlo, devn);
      break;
    case 64:
      k_vo_refine<64><<<nitems, 256, 0, s>>>(Xf, permf, nfit, center.as<float>(), rad.as<float>(), nct, nmax,
                                             rowthr, dlo, devn);
      break;
    case 96:
      k_vo_refine<96><<<nitems, 256, 0, s>>>(Xf, permf, nfit, center.as<float>(), rad.as<float>(), nct, nmax,
                                             rowthr, dlo, devn);
      break;
    case 128:
      k_vo_refine<128><<<nitems, 256, 0, s>>>(Xf, permf, nfit, center.as<float>(), rad.as<float>(), nct, nmax,
                                              rowthr, dlo, devn);
      break;
    default:
      return mds_fail(ctx, MDS_ERR_INTERNAL, "vec_tile_bounds: padded dimension %d", Dp);
  }
  ctx->stats.launches++;
  if (tdseg) {
    k_vo_start<<<dim3(nitems, nseg), 32, 0, s>>>(dlo, nct, nseg, tdseg, nullptr, 0);
    ctx->stats.launches++;
  }
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// Threshold seeds of the sorted fit rows (k_vo_seed_rows) into rowthr, whose
// entries are +inf-like before (a row without a seed keeps its value). The
// reference set is in tiles of 128.
int vec_seed_rows(mds_ctx* ctx, const float* Xr, const int* permr, int nref, const float* Xf, const int* permf,
                  int nfit, int Dp, const int* tdall, int k1, const float* nmax, float* rowthr,
                  const unsigned* devn) {
  if (k1 > 128) return MDS_OK;
  const int ncoltiles = (nref + 127) / 128, nitems = (nfit + 255) / 256;
  const size_t smem = sizeof(float) * ((size_t)128 * (Dp + 1) + 8 * (size_t)Dp);
  static bool attr_done = false;
  static size_t attr_limit = 0;
  MDS_TRY(mds_allow_dyn_smem(ctx, k_vo_seed_rows, &attr_done, &attr_limit));
  if (smem > attr_limit) return MDS_OK;
  k_vo_seed_rows<<<nitems, 256, smem, ctx->stream>>>(Xr, permr, nref, Xf, permf, nfit, Dp, tdall, ncoltiles, k1,
                                                      nmax, rowthr, devn);
  ctx->stats.launches++;
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// dst[perm[i]] = src[i]: a per-row array of the sorted set back in the
// original order.
int vec_unsort(mds_ctx* ctx, const float* src, const int* perm, int n, float* dst) {
  k_vo_unsort<<<(n + 255) / 256, 256, 0, ctx->stream>>>(src, perm, n, dst);
  ctx->stats.launches++;
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}
