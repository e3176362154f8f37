// knn_rms.cu -- all-pairs minimum-RMSD k-nearest neighbours on sm_103a.
//
// Replaces the compute core of knn_rms.cpp (distance() :38-41, the centring
// :186-206 and the OpenMP row loop with permutation::sort(k+1) :213-293).
//
// Pipeline (all on ctx->stream):
//  1. k_center      reset_x centring (knn_rms.cpp:189,199) of the first
//                   reference frame, from which the template mu (that frame
//                   in its principal axes) is built; coordinates scaled by
//                   sqrt(w/M) so that every sum below is per unit mass;
//                   layout [frame][xyz][Ap] float (atom-major, Ap = natoms
//                   rounded up to 64, zero padded).
//  2. k_prep_sums, k_prep_rot, k_prep_out
//                   centre every frame and superpose it once onto mu, store
//                   deviations a = R y - mu and the per-frame screen record.
//  3. screen        all pairs: deviation Gram + shifted QCP lower bound of
//                   RMSD^2, fused per-row top-K' (never an N x N matrix).
//                   FP32 CUDA cores (k_screen_fp32) or tcgen05 split BF16
//                   (knn_rms_tc.cu).
//  4. k_recheck     merge the per-segment candidate lists, recompute every
//                   candidate exactly the way the reference does (optimal
//                   rotation, then the RMSD of the rotated coordinates),
//                   select k+1, drop position 0, verify the guard.
//  5. rows whose guard failed are screened again with 4x the candidates.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <vector>

#include "knn_common.cuh"
#include "qcp.cuh"

// ---------------------------------------------------------------------------
// 1. centring
// ---------------------------------------------------------------------------
// Block sum of N float partials: FP32 shuffle tree inside each warp (FP64
// issues at a small fraction of the FP32 rate on this GPU), then the warps'
// sums added in FP64 in warp order. red holds (blockDim/32) * N doubles.
// red holds (blockDim/32 + 1) * N doubles; thread i < N forms sum i (the
// only FP64 work) and every thread reads the N sums back.
template <int N>
__device__ __forceinline__ void block_sum_vecf(const float (&p)[N], double (&out)[N], double* red) {
  float v[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    v[i] = p[i];
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) red[w * N + i] = (double)v[i];
  __syncthreads();
  if (threadIdx.x < N) {
    double s = 0;
    for (int j = 0; j < nw; ++j) s += red[j * N + threadIdx.x];
    red[nw * N + threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = red[nw * N + i];
  __syncthreads();
}

// Block sum of N float partials entirely in FP32 (shuffle tree per warp, then
// the warps' sums added in warp order by thread i < N). For the prep sums,
// whose accuracy only sets how close the pre-alignment rotation is to the
// optimum; a conversion or add on the FP64 pipe costs a whole warp's issue on
// this GPU. red holds (blockDim/32 + 1) * N floats.
template <int N>
__device__ __forceinline__ void block_sum_vec32(const float (&p)[N], float (&out)[N], float* red) {
  float v[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    v[i] = p[i];
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) red[w * N + i] = v[i];
  __syncthreads();
  if (threadIdx.x < N) {
    float s = 0.f;
    for (int j = 0; j < nw; ++j) s += red[j * N + threadIdx.x];
    red[nw * N + threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = red[nw * N + i];
  __syncthreads();
}

// Double-float accumulation (hi + lo, an unevaluated sum): products by an
// FMA-exact TwoProduct, additions by Knuth's TwoSum. The _rn intrinsics keep
// the compiler from contracting the steps into FMAs, which would break the
// error terms.
__device__ __forceinline__ void df_add(float& hi, float& lo, float bh, float bl) {
  const float t = __fadd_rn(hi, bh);
  const float z = __fsub_rn(t, hi);
  const float te = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(bh, z));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(te, bl));
}
__device__ __forceinline__ void df_add_prod(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  df_add(hi, lo, p, fmaf(a, b, -p));
}
// The 9 sums U[3c+d] = sum_atoms a_c mu_d of a frame as double-float pairs,
// over the block: out[2i] = hi, out[2i+1] = lo of U[i] (thread 0; red holds
// (blockDim/32) * 18 floats). Their differences between two frames,
// sum mu (a_i - a_j)^T, cancel to the size of the frames' difference, so they
// are kept to about 2^-48 relative.
__device__ __forceinline__ void block_sum_df9(float (&h)[9], float (&l)[9], float* red, float* out) {
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < 9; ++i)
    for (int o = 16; o > 0; o >>= 1) {
      const float bh = __shfl_xor_sync(0xffffffffu, h[i], o), bl = __shfl_xor_sync(0xffffffffu, l[i], o);
      df_add(h[i], l[i], bh, bl);
    }
  __syncthreads();
  if (ln == 0)
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      red[w * 18 + 2 * i] = h[i];
      red[w * 18 + 2 * i + 1] = l[i];
    }
  __syncthreads();
  if (threadIdx.x < 9) {
    const int i = threadIdx.x;
    float sh = red[2 * i], sl = red[2 * i + 1];
    for (int j = 1; j < nw; ++j) df_add(sh, sl, red[j * 18 + 2 * i], red[j * 18 + 2 * i + 1]);
    const float t = __fadd_rn(sh, sl);  // renormalise: hi = fl(hi + lo)
    out[2 * i] = t;
    out[2 * i + 1] = __fsub_rn(sl, __fsub_rn(t, sh));
  }
  __syncthreads();
}

// Block sum of N values at once: every warp reduces its N partial sums with
// shuffles, lane 0 stores them in red[warp * N + i], one barrier, then every
// thread adds the warps' rows in order. red holds (blockDim/32) * N doubles.
template <int N>
__device__ __forceinline__ void block_sum_vec(double (&v)[N], double* red) {
#pragma unroll
  for (int i = 0; i < N; ++i)
    for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) red[w * N + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) {
    double s = 0;
    for (int j = 0; j < nw; ++j) s += red[j * N + i];
    v[i] = s;
  }
  __syncthreads();
}

// One block per frame. raw: [n][natoms][3]; out: [n][3][Ap]; E: |y|^2 per
// unit mass (double). tm: float sum of masses in file order (reset_x's tm).
// Per-atom arithmetic is FP32 (FP64 issues at a small fraction of the FP32
// rate on this GPU); only the block reductions of the per-thread partial sums
// are FP64. The centre of mass therefore differs from reset_x's FP64 sum by
// ~1e-7 relative, which moves an optimal-superposition RMSD only at second
// order (the cross term vanishes for centred frames).
__global__ void k_center(const float* __restrict__ raw, int n, int natoms, int Ap,
                         const float* __restrict__ mass, const float* __restrict__ swn, float tm,
                         float* __restrict__ out, double* __restrict__ E) {
  __shared__ double red[32 * 3];
  int f = blockIdx.x;
  if (f >= n) return;
  const float* x = raw + (int64_t)f * natoms * 3;
  float p[3] = {0.f, 0.f, 0.f};
  for (int a = threadIdx.x; a < natoms; a += blockDim.x) {
    float mm = mass[a];
    for (int c = 0; c < 3; ++c) p[c] = fmaf(mm, x[3 * a + c], p[c]);
  }
  double s[3] = {p[0], p[1], p[2]};
  block_sum_vec<3>(s, red);
  float com[3];
  for (int c = 0; c < 3; ++c) com[c] = (float)(s[c] / (double)tm);
  float e = 0.f;
  float* o = out + (int64_t)f * 3 * Ap;
  for (int a = threadIdx.x; a < Ap; a += blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      float v = 0.0f;
      if (a < natoms) {
        v = (x[3 * a + c] - com[c]) * swn[a];
        e = fmaf(v, v, e);
      }
      o[c * Ap + a] = v;
    }
  }
  double ev[1] = {e};
  block_sum_vec<1>(ev, red);
  if (threadIdx.x == 0) E[f] = ev[0];
}

// ---------------------------------------------------------------------------
// 2. centring and superposition onto the template, in three kernels
// ---------------------------------------------------------------------------
// The centred, mass-scaled coordinates y = (x - com) sqrt(w/M) of a frame are
// recomputed from the raw frame in each pass, so only the deviations
// a = R y - mu [n][3][Ap] and the screen records [n][MDS_REC] are written.
// The rotation only has to be a proper rotation (x~ = mu + a is an exact
// rigid copy of the frame for any R; a better fit only makes |a| smaller), so
// the per-atom work is FP32 with FP64 sums across warps. The quaternion is
// solved in FP64 by one thread per frame in a kernel of its own, so the
// per-atom kernels keep few registers and many frames in flight per SM.
// Between the kernels the record row carries com (0..2) and the sums of the
// rotation fit (3..12, then R in 3..11).

// Pass 1 + 2 (one block per frame): centre of mass, then |y|^2 and the
// covariance sum y mu^T.
// bad (optional): receives the smallest index (fbase + f) of a frame with a
// non-finite coordinate.
__global__ void __launch_bounds__(128) k_prep_sums(const float* __restrict__ raw, int n, int natoms, int Ap,
                                                   const float* __restrict__ mass, const float* __restrict__ swn,
                                                   float tm, const float* __restrict__ mu, int nofit,
                                                   float* __restrict__ rec, int* __restrict__ bad, int fbase) {
  __shared__ float red[5 * 10];
  const int f = blockIdx.x;
  if (f >= n) return;
  const float* x = raw + (int64_t)f * natoms * 3;
  float com[3];
  {
    float p[3] = {0.f, 0.f, 0.f};
    bool fin = true;
#pragma unroll 4
    for (int a = threadIdx.x; a < natoms; a += blockDim.x) {
      const float mm = mass[a];
      for (int c = 0; c < 3; ++c) {
        const float v = x[3 * a + c];
        fin &= isfinite(v);
        p[c] = fmaf(mm, v, p[c]);
      }
    }
    if (bad && __syncthreads_or(!fin) && threadIdx.x == 0) atomicMin(bad, fbase + f);
    float sc[3];
    block_sum_vec32<3>(p, sc, red);
    for (int c = 0; c < 3; ++c) com[c] = sc[c] / tm;
  }
  float* r = rec + (int64_t)f * MDS_REC;
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; ++c) r[c] = com[c];
  if (nofit) return;
  float p[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // |y|^2, sum y mu^T
#pragma unroll 2
  for (int a = threadIdx.x; a < natoms; a += blockDim.x) {
    const float w = swn[a];
    float yc[3], mc[3] = {mu[a], mu[Ap + a], mu[2 * Ap + a]};
    for (int c = 0; c < 3; ++c) yc[c] = (x[3 * a + c] - com[c]) * w;
    p[0] = fmaf(yc[0], yc[0], fmaf(yc[1], yc[1], fmaf(yc[2], yc[2], p[0])));
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) p[1 + 3 * c + d] = fmaf(yc[c], mc[d], p[1 + 3 * c + d]);
  }
  float sv[10];
  block_sum_vec32<10>(p, sv, red);
  if (threadIdx.x == 0)
    for (int i = 0; i < 10; ++i) r[3 + i] = sv[i];
}

// The rotation of every frame (one thread per frame, FP64 QCP): record
// entries 3..12 (|y|^2, y mu^T) -> 3..11 (R, row-major).
__global__ void k_prep_rot(int n, const double* __restrict__ M0, float* __restrict__ rec) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n) return;
  float* r = rec + (int64_t)f * MDS_REC;
  double S[9], R[9];
  for (int i = 0; i < 9; ++i) S[i] = r[4 + i];
  qcp_rotation_fp64(S, 0.5 * ((double)r[3] + M0[0] + M0[4] + M0[8]), R);
  for (int i = 0; i < 9; ++i) r[3 + i] = (float)R[i];
}

// Pass 3 (one block per frame): deviations a = R y - mu and the record sums
// (|a|^2, a mu^T with the template's M0), which replace the record row.
__global__ void __launch_bounds__(128) k_prep_out(const float* __restrict__ raw, int n, int natoms, int Ap,
                                                  const float* __restrict__ swn, const float* __restrict__ mu,
                                                  const double* __restrict__ M0, int nofit, float* __restrict__ dev,
                                                  float* __restrict__ rec, float* __restrict__ uhl) {
  __shared__ float red[5 * 10];
  __shared__ float redu[4 * 18];
  const int f = blockIdx.x;
  if (f >= n) return;
  const float* x = raw + (int64_t)f * natoms * 3;
  float* r = rec + (int64_t)f * MDS_REC;
  const float com[3] = {r[0], r[1], r[2]};
  float R[9];
  for (int i = 0; i < 9; ++i) R[i] = nofit ? ((i % 4 == 0) ? 1.0f : 0.0f) : r[3 + i];
  float ea = 0.f, u[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float uh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ul[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float* o = dev + (int64_t)f * 3 * Ap;
#pragma unroll 2
  for (int a = threadIdx.x; a < Ap; a += blockDim.x) {
    if (a < natoms) {
      const float w = swn[a];
      float yc[3], mc[3] = {mu[a], mu[Ap + a], mu[2 * Ap + a]}, av[3];
      for (int c = 0; c < 3; ++c) yc[c] = (x[3 * a + c] - com[c]) * w;
      for (int c = 0; c < 3; ++c) {
        const float ry = fmaf(R[3 * c], yc[0], fmaf(R[3 * c + 1], yc[1], R[3 * c + 2] * yc[2]));
        av[c] = ry - mc[c];
        o[c * Ap + a] = av[c];
      }
      for (int c = 0; c < 3; ++c) {
        ea = fmaf(av[c], av[c], ea);
        for (int d = 0; d < 3; ++d) u[3 * c + d] = fmaf(av[c], mc[d], u[3 * c + d]);
      }
      if (uhl)
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d) df_add_prod(uh[3 * c + d], ul[3 * c + d], av[c], mc[d]);
    } else {
      for (int c = 0; c < 3; ++c) o[c * Ap + a] = 0.0f;
    }
  }
  if (uhl) block_sum_df9(uh, ul, redu, uhl + (int64_t)f * 18);  // uniform branch: all threads or none
  const float eup[10] = {ea, u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8]};
  float eu[10];
  block_sum_vec32<10>(eup, eu, red);  // every thread has read the record row before this barrier
  if (threadIdx.x == 0) {
    // the template's M0 in FP64 once per frame (one thread)
    const float* U = eu + 1;
    const float sxx = U[0], syy = U[4], szz = U[8];
    const float sxy = 0.5f * (U[1] + U[3]), sxz = 0.5f * (U[2] + U[6]), syz = 0.5f * (U[5] + U[7]);
    r[0] = (float)(M0[0] + sxx);
    r[1] = (float)(M0[4] + syy);
    r[2] = (float)(M0[8] + szz);
    r[3] = (float)(0.5 * (M0[1] + M0[3]) + sxy);
    r[4] = (float)(0.5 * (M0[2] + M0[6]) + sxz);
    r[5] = (float)(0.5 * (M0[5] + M0[7]) + syz);
    r[6] = sxx; r[7] = syy; r[8] = szz;
    r[9] = sxy; r[10] = sxz; r[11] = syz;
    r[12] = U[5] - U[7];
    r[13] = U[6] - U[2];
    r[14] = U[1] - U[3];
    r[15] = eu[0];
  }
}

// ---------------------------------------------------------------------------
// 3. FP32 CUDA-core screen: tile of 32 fit x 64 ref frames per step, each
//    thread owns 2 x 4 pairs (72 accumulators), atoms staged through shared
//    memory in chunks of 32 with cp.async double buffering.
// ---------------------------------------------------------------------------
#define SC_TM 32
#define SC_TN 64
#define SC_KC 32
#define SC_FS 98  // floats per frame per stage: 3*32 + 2 (bank spread)
#define SC_THREADS 256

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Column tiles of a segment [t0, t1) visited outward from tile td (td,
// td+1, td-1, ...): for a set screened against itself td holds the row
// tile's own frames, so a row's threshold tightens early.
__device__ __forceinline__ int sc_tile_order(int i, int t0, int t1, int td) {
  const int L = td - t0, Rn = t1 - 1 - td, m = min(L, Rn);
  if (i == 0) return td;
  if (i <= 2 * m) return (i & 1) ? td + (i + 1) / 2 : td - i / 2;
  const int j = i - 2 * m;
  return (Rn > L) ? td + m + j : td - m - j;
}

__global__ void __launch_bounds__(SC_THREADS, 1)
k_screen_fp32(const float* __restrict__ Af, const float* __restrict__ Ar,
              const float* __restrict__ recf, const float* __restrict__ recr, int nrows,
              const int* __restrict__ rowlist, int Nr, int Ap, int nofit, float guard, int Kp,
              int nseg, uint64_t* __restrict__ cand, int* __restrict__ cand_n, const Fp32ScreenExtra ex) {
  // Tile skipping (ex.pivlb != null, a set screened against itself): the
  // tensor-core screen's row-tile pivots (the middle frame of every 40-frame
  // tile) and 80-frame column tiles. RMSD is a metric, so for row i and any
  // frame j of 80-frame tile T, RMSD(i, j) >= max over the pivots p of T's
  // two row tiles of lb(i, p) - r_T(p), and >= rowlo[R(i)][T]. A 64-frame
  // tile of this screen overlaps one or two 80-frame tiles; the smaller of
  // their bounds holds for all its frames. The tile is skipped when every
  // row has that bound L > 0 with L^2 above its threshold.
  // Shared row thresholds (ex.rowthr): each compaction lowers rowthr[row]
  // (atomicMin on the float's bits, values >= 0), and every segment appends
  // only below min(own threshold, rowthr) and skips by it.
  // Thresholds from the (k+1)-th bound (ex.nmax): a bound b is the screen
  // value minus the guard g (|a_i|^2 + |a_j|^2), and the screen value is
  // within the guard of the exact RMSD^2, so the row's (k+1)-th exact value
  // is at most b_(k+1) + 2 g (|a_i|^2 + nmax); a compaction sets the row
  // threshold to the smaller of that and the K'-th bound, and the first one
  // runs as soon as k1 keys have arrived.
  // Dense mode (ex.dense != null; the pivot pass of this screen): every
  // pair's lower bound of RMSD (sqrt of the bound of RMSD^2) is written to
  // dense[j][i] (j: reference frame); no lists.
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sfit = reinterpret_cast<float*>(smem_raw);                 // [2][32*98]
  float* sref = sfit + 2 * SC_TM * SC_FS;                           // [2][64*98]
  float* scol = sref + 2 * SC_TN * SC_FS;                           // [64][16]
  int* scnt = reinterpret_cast<int*>(scol + SC_TN * MDS_REC);       // [32]
  float* sthr = reinterpret_cast<float*>(scnt + SC_TM);             // [32]
  uint64_t* pool = reinterpret_cast<uint64_t*>(sthr + SC_TM);       // [32][P2]
  __shared__ float sgthr[SC_TM];  // the rows' shared thresholds, read per tile
  // a row's pool holds its K' best plus one tile of new entries; its stride
  // is the power of two the sort works on
  const int P2 = next_pow2(Kp + SC_TN);

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int lane = tid & 31, warp = tid >> 5;
  const int rt = blockIdx.x / nseg, seg = blockIdx.x % nseg;
  const int row0 = rt * SC_TM;
  // column segment [c0, c1) in whole tiles
  const int ntiles = (Nr + SC_TN - 1) / SC_TN;
  const int t0 = (int)((int64_t)ntiles * seg / nseg), t1 = (int)((int64_t)ntiles * (seg + 1) / nseg);
  const int td = ex.diag ? min(max((row0 + SC_TM / 2) / SC_TN, t0), max(t1 - 1, t0)) : t0;
  const bool dense = ex.dense != nullptr;
  const float INF = __int_as_float(0x7f800000);

  int grow[2];
  float rrec[2][MDS_REC];
  for (int p = 0; p < 2; ++p) {
    int lr = row0 + ty + 16 * p;
    grow[p] = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
    for (int i = 0; i < MDS_REC; ++i) rrec[p][i] = (grow[p] >= 0) ? recf[(int64_t)grow[p] * MDS_REC + i] : 0.f;
  }
  if (tid < SC_TM) {
    scnt[tid] = 0;
    sthr[tid] = INF;
  }
  const int nchunks = Ap / SC_KC;

  auto load_chunk = [&](int stage, int tile, int kc) {
    float* df = sfit + stage * SC_TM * SC_FS;
    float* dr = sref + stage * SC_TN * SC_FS;
    // fit: 32 frames x 3 coords x 16 pairs of floats
    for (int e = tid; e < SC_TM * 3 * 16; e += SC_THREADS) {
      int fr = e / 48, rem = e % 48, c = rem / 16, h = rem % 16;
      int lr = row0 + fr;
      int g = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
      const float* src = Af + ((int64_t)(g < 0 ? 0 : g) * 3 + c) * Ap + kc * SC_KC + 2 * h;
      cp_async8(df + fr * SC_FS + c * SC_KC + 2 * h, src, g >= 0);
    }
    for (int e = tid; e < SC_TN * 3 * 16; e += SC_THREADS) {
      int fr = e / 48, rem = e % 48, c = rem / 16, h = rem % 16;
      int j = tile * SC_TN + fr;
      const float* src = Ar + ((int64_t)(j < Nr ? j : 0) * 3 + c) * Ap + kc * SC_KC + 2 * h;
      cp_async8(dr + fr * SC_FS + c * SC_KC + 2 * h, src, j < Nr);
    }
  };

  for (int ti = 0; ti < t1 - t0; ++ti) {
    const int tile = ex.diag ? sc_tile_order(ti, t0, t1, td) : t0 + ti;
    __syncthreads();
    // the rows' shared thresholds now (they only decrease)
    if (tid < SC_TM) {
      const int lr = row0 + tid;
      const int g = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
      sgthr[tid] = (ex.rowthr && g >= 0) ? __ldcg(ex.rowthr + g) : INF;
    }
    if (ex.pivlb && !dense) {
      // skip test: one lane per row
      bool can = true;
      if (tid < SC_TM) {
        const int lr = row0 + tid;
        const int g = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
        if (g >= 0) {
          const float thr = fminf(sthr[tid], __ldcg(ex.rowthr + g));
          const int jlo = tile * SC_TN, jhi = min(jlo + SC_TN, Nr) - 1;
          const int Ta = jlo / TC_FR_N, Tb = jhi / TC_FR_N;
          const int R = g / TC_FR_M;
          float L = INF;
          for (int T = Ta; T <= Tb; ++T) {
            const int pa = 2 * T;
            float LT = __ldg(ex.rowlo + (int64_t)R * ex.nC + T);
            LT = fmaxf(LT, __ldg(ex.pivlb + (int64_t)pa * ex.nfit + g) - __ldg(ex.prad + pa));
            if (pa + 1 < ex.nR) LT = fmaxf(LT, __ldg(ex.pivlb + (int64_t)(pa + 1) * ex.nfit + g) - __ldg(ex.prad + pa + 1));
            L = fminf(L, LT);
          }
          can = L > 0.0f && L * L > thr;
        }
      }
      if (__syncthreads_and(can)) continue;
    }
    if (ex.ntiles && !dense && tid == 0) atomicAdd(ex.ntiles, 1ull);
    // column records of this tile
    for (int e = tid; e < SC_TN * MDS_REC; e += SC_THREADS) {
      int fr = e / MDS_REC, i = e % MDS_REC;
      int j = tile * SC_TN + fr;
      scol[e] = (j < Nr) ? recr[(int64_t)j * MDS_REC + i] : 0.f;
    }
    float acc[2][4][9];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int i = 0; i < 9; ++i) acc[p][q][i] = 0.f;

    load_chunk(0, tile, 0);
    cp_async_commit();
    for (int kc = 0; kc < nchunks; ++kc) {
      if (kc + 1 < nchunks) {
        load_chunk((kc + 1) & 1, tile, kc + 1);
        cp_async_commit();
        cp_async_wait1();
      } else {
        cp_async_wait0();
      }
      __syncthreads();
      const float* df = sfit + (kc & 1) * SC_TM * SC_FS;
      const float* dr = sref + (kc & 1) * SC_TN * SC_FS;
#pragma unroll 2
      for (int a = 0; a < SC_KC; a += 2) {
        float2 fv[2][3], rv[4][3];
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            fv[p][c] = *reinterpret_cast<const float2*>(df + (ty + 16 * p) * SC_FS + c * SC_KC + a);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            rv[q][c] = *reinterpret_cast<const float2*>(dr + (tx + 16 * q) * SC_FS + c * SC_KC + a);
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                acc[p][q][3 * c + d] = fmaf(fv[p][c].x, rv[q][d].x, acc[p][q][3 * c + d]);
                acc[p][q][3 * c + d] = fmaf(fv[p][c].y, rv[q][d].y, acc[p][q][3 * c + d]);
              }
      }
      __syncthreads();
    }
    // epilogue: lower bounds and top-K' insertion (or the dense bounds)
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      if (grow[p] < 0) continue;
      int lr = ty + 16 * p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int j = tile * SC_TN + tx + 16 * q;
        if (j >= Nr) continue;
        const float* cr = scol + (tx + 16 * q) * MDS_REC;
        const float thr = dense ? INF : fminf(sthr[lr], sgthr[lr]);
        float s = screen_shifted_f32(acc[p][q], rrec[p], cr, nofit != 0, guard * (rrec[p][15] + cr[15]), thr);
        s = fmaxf(s, 0.0f);
        if (dense) {
          ex.dense[(int64_t)j * nrows + row0 + lr] = sqrtf(s);
        } else if (s < thr) {
          int pos = atomicAdd(&scnt[lr], 1);
          pool[lr * P2 + pos] = mds_pack_key(s, j);
        }
      }
    }
    __syncthreads();
    if (dense) continue;
    // compaction of rows whose pool exceeds K' (or first holds k1 keys)
    for (int r = warp; r < SC_TM; r += SC_THREADS / 32) {
      const int n = scnt[r];
      const bool first = ex.nmax && sthr[r] == INF && n >= ex.k1;
      if (n <= Kp && !first) continue;
      warp_bitonic_sort(pool + r * P2, n, P2, lane);
      if (lane == 0) {
        float t = (n >= Kp) ? mds_key_value(pool[r * P2 + Kp - 1]) : INF;
        const int lr = row0 + r;
        const int g = (lr < nrows) ? (rowlist ? rowlist[lr] : lr) : -1;
        if (ex.nmax && g >= 0)
          t = fminf(t, mds_key_value(pool[r * P2 + ex.k1 - 1]) +
                           2.0f * guard * (__ldg(recf + (int64_t)g * MDS_REC + 15) + __ldg(ex.nmax)));
        scnt[r] = min(n, Kp);
        sthr[r] = t;
        if (ex.rowthr && g >= 0) atomicMin(reinterpret_cast<int*>(ex.rowthr + g), __float_as_int(t));
      }
      __syncwarp();
    }
  }
  if (dense) return;
  __syncthreads();
  // final: sort each row's pool and write it out
  for (int r = warp; r < SC_TM; r += SC_THREADS / 32) {
    int lr = row0 + r;
    if (lr >= nrows) continue;
    int n = min(scnt[r], Kp);
    warp_bitonic_sort(pool + r * P2, scnt[r], P2, lane);
    uint64_t* dst = cand + ((int64_t)lr * nseg + seg) * Kp;
    for (int x = lane; x < n; x += 32) dst[x] = pool[r * P2 + x];
    if (lane == 0) cand_n[(int64_t)lr * nseg + seg] = n;
  }
}

size_t screen_fp32_smem(int Kp) {
  return sizeof(float) * (2 * SC_TM * SC_FS + 2 * SC_TN * SC_FS + SC_TN * MDS_REC) +
         sizeof(int) * SC_TM + sizeof(float) * SC_TM + sizeof(uint64_t) * SC_TM * next_pow2(Kp + SC_TN);
}

int launch_screen_fp32(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Af, const float* Ar,
                       const float* recf, const float* recr, int nrows, const int* rowlist, int Kp,
                       int nseg, uint64_t* cand, int* cand_n, const Fp32ScreenExtra* extra) {
  size_t smem = screen_fp32_smem(Kp);
  static bool attr_set = false;  // once: launches may also happen while a stream is captured
  static size_t limit = 0;
  MDS_TRY(mds_allow_dyn_smem(ctx, k_screen_fp32, &attr_set, &limit));
  if (smem > limit) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "screen shared memory %zu > %zu", smem, limit);
  int nrt = (nrows + SC_TM - 1) / SC_TM;
  ctx->stats.launches++;
  k_screen_fp32<<<nrt * nseg, SC_THREADS, smem, ctx->stream>>>(
      Af, Ar, recf, recr, nrows, rowlist, pl.nref, pl.Ap, pl.nofit, pl.guard_fp32, Kp, nseg, cand, cand_n,
      extra ? *extra : Fp32ScreenExtra{});
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// ---------------------------------------------------------------------------
// 4. merge + exact recheck + selection + output
// ---------------------------------------------------------------------------
#define RC_THREADS 256
#define RC_CHUNK 128
#define RC_GW 8  // lanes per candidate in the recheck's atom loop (32 / RC_GW candidates per warp)

// Exact RMSD (nm) of fit frame (in shared memory) vs reference frame j for a
// chunk of candidates: covariance per warp, FP64 rotation per thread, then
// the RMSD of the rotated fit frame against the reference frame.
// Exact RMSD of the fit frame against nc reference frames cj[], one warp per
// pair, in one pass over the atoms. With x~ = mu + a the superposed copies
// (rigid copies of the frames) and d = a_i - a_j = x~_i - x~_j:
//   D = sum |d|^2,  S = sum x~_i x~_j^T = C_i - P,  P = sum x~_i d^T,
// C_i = sum x~_i x~_i^T (per row, precomputed). D is a sum of positive
// terms, and P's antisymmetric part (the small vector b of the key matrix)
// is formed from the small d, so FP32 keeps them accurate; RMSD^2 = D - 2 nu
// (qcp.cuh: shifted_rmsd2_f32). sa = a_i, sx = x~_i (shared memory), C6 =
// (Cxx, Cyy, Czz, Cxy, Cxz, Cyz).
// RMSD^2 of a pair from its sums w = (D, Q[9]) (see recheck_chunk), the fit
// row's C6 and U (ui, double-float pairs) and the reference frame's U (uj).
__device__ __forceinline__ float pair_rmsd2(const float* w, const float* C6, const float* ui,
                                           const float* __restrict__ uj, bool nofit) {
  if (nofit) return w[0];
  // P[3r+s] = sum x~_r d_s = Q[3r+s] + sum mu_r d_s, and
  // sum mu_r d_s = U_i[3s+r] - U_j[3s+r] from the frames' double-float U
  float P[9];
#pragma unroll
  for (int rr = 0; rr < 3; ++rr)
#pragma unroll
    for (int ss = 0; ss < 3; ++ss) {
      const int iu = 3 * ss + rr;
      float dh = ui[2 * iu], dl = ui[2 * iu + 1];
      df_add(dh, dl, -__ldg(uj + 2 * iu), -__ldg(uj + 2 * iu + 1));
      P[3 * rr + ss] = w[1 + 3 * rr + ss] + (dh + dl);
    }
  return shifted_rmsd2_f32(w[0], C6[0] - P[0], C6[1] - P[4], C6[2] - P[8], 2.0f * C6[3] - (P[1] + P[3]),
                           2.0f * C6[4] - (P[2] + P[6]), 2.0f * C6[5] - (P[5] + P[7]), P[7] - P[5], P[2] - P[6],
                           P[3] - P[1]);
}

// The sums of one pair over four atoms: D += |d|^2 and Q[3r+s] += a_i,r d_s
// (unless nofit), d = a_i - a_j; x* = a_i's and y* = a_j's x, y, z of the
// four atoms, two atoms per packed instruction.
__device__ __forceinline__ void pair_acc4(float2 (&w)[10], const float4& ia, const float4& ib, const float4& ic,
                                          const float4& ja, const float4& jb, const float4& jc, bool nofit) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 x0[2] = {make_float2(ia.x, ia.y), make_float2(ia.z, ia.w)};
  const float2 x1[2] = {make_float2(ib.x, ib.y), make_float2(ib.z, ib.w)};
  const float2 x2[2] = {make_float2(ic.x, ic.y), make_float2(ic.z, ic.w)};
  const float2 y0[2] = {make_float2(ja.x, ja.y), make_float2(ja.z, ja.w)};
  const float2 y1[2] = {make_float2(jb.x, jb.y), make_float2(jb.z, jb.w)};
  const float2 y2[2] = {make_float2(jc.x, jc.y), make_float2(jc.z, jc.w)};
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float2 d0 = __ffma2_rn(y0[e], m1, x0[e]), d1 = __ffma2_rn(y1[e], m1, x1[e]);
    const float2 d2 = __ffma2_rn(y2[e], m1, x2[e]);
    w[0] = __ffma2_rn(d0, d0, __ffma2_rn(d1, d1, __ffma2_rn(d2, d2, w[0])));
    if (!nofit) {
      w[1] = __ffma2_rn(x0[e], d0, w[1]); w[2] = __ffma2_rn(x0[e], d1, w[2]); w[3] = __ffma2_rn(x0[e], d2, w[3]);
      w[4] = __ffma2_rn(x1[e], d0, w[4]); w[5] = __ffma2_rn(x1[e], d1, w[5]); w[6] = __ffma2_rn(x1[e], d2, w[6]);
      w[7] = __ffma2_rn(x2[e], d0, w[7]); w[8] = __ffma2_rn(x2[e], d1, w[8]); w[9] = __ffma2_rn(x2[e], d2, w[9]);
    }
  }
}

__device__ void recheck_chunk(const float* __restrict__ sa, const float* __restrict__ ui, const float* C6,
                              const float* __restrict__ Ar, const float* __restrict__ Ur, int Ap, const int* cj,
                              int nc, bool nofit, float* sd, float* ssum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // A warp takes 32 / RC_GW candidates at a time, RC_GW lanes each; four
  // atoms per lane and load (Ap is a multiple of 64; padding atoms are zero
  // in a_i and a_j, so they add nothing). Per candidate: D = sum |d|^2 and
  // Q[3r+s] = sum a_i,r d_s with d = a_i - a_j; the row's deviations are the
  // only shared-memory reads. A 128-bit shared load costs one wavefront per
  // quarter warp however many groups read the same address, so more, narrower
  // groups share each load of the row among more candidates.
  constexpr int CPW = 32 / RC_GW;
  const int grp = lane / RC_GW, gl = lane % RC_GW;
  const int Ap4 = Ap >> 2;
  const float4* sa4 = reinterpret_cast<const float4*>(sa);
  for (int c0 = CPW * warp; c0 < nc; c0 += CPW * nw) {
    const int c = c0 + grp;
    const bool valid = c < nc;
    const float4* aj4 = reinterpret_cast<const float4*>(Ar + (int64_t)cj[valid ? c : c0] * 3 * Ap);
    // Packed FP32 arithmetic (two atoms per instruction, each lane keeping
    // two partial sums per quantity). (Two candidates per group, sharing each
    // load of the row, needed 128 registers and ran slower at half the
    // occupancy: 3.25 against 2.42 ms at 20,000 x 1,000.)
    float2 w[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) w[i] = make_float2(0.0f, 0.0f);
    for (int q = gl; q < Ap4; q += RC_GW) {
      const float4 ia = sa4[q], ib = sa4[Ap4 + q], ic = sa4[2 * Ap4 + q];
      const float4 ja = __ldg(aj4 + q), jb = __ldg(aj4 + Ap4 + q), jc = __ldg(aj4 + 2 * Ap4 + q);
      pair_acc4(w, ia, ib, ic, ja, jb, jc, nofit);
    }
    float v[10];
#pragma unroll
    for (int i = 0; i < 10; ++i) v[i] = w[i].x + w[i].y;
    // sums over the lanes of each group (one shuffle serves every group)
#pragma unroll
    for (int i = 0; i < 10; ++i)
      for (int o = RC_GW / 2; o > 0; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    if (valid && gl == 0) {
      float2* w2 = reinterpret_cast<float2*>(ssum + c * 10);
#pragma unroll
      for (int i = 0; i < 5; ++i) w2[i] = make_float2(v[2 * i], v[2 * i + 1]);
    }
  }
  __syncthreads();
  // the eigenvalue solves, one pair per thread
  for (int c = threadIdx.x; c < nc; c += blockDim.x)
    sd[c] = sqrtf(fmaxf(pair_rmsd2(ssum + c * 10, C6, ui, Ur + (int64_t)cj[c] * 18, nofit), 0.0f));
  __syncthreads();
}

// C6 = sum x~ x~^T of a fit row (x~ = mu + a_i), and its U = sum a_i mu^T as
// double-float pairs (ui[2i], ui[2i+1]), the same sums as the reference
// frames' Ur. Called by the whole block; C6 and ui in shared memory.
__device__ void row_constants(const float* __restrict__ af, const float* __restrict__ mu, int Ap, int natoms,
                              int nofit, float* C6, float* ui, double* s_red, float* redu) {
  float p[6] = {0, 0, 0, 0, 0, 0};
  float uh[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ul[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int a = threadIdx.x; a < natoms; a += blockDim.x) {
    const float m[3] = {mu[a], mu[Ap + a], mu[2 * Ap + a]}, av[3] = {af[a], af[Ap + a], af[2 * Ap + a]};
    const float x0 = m[0] + av[0], x1 = m[1] + av[1], x2 = m[2] + av[2];
    p[0] = fmaf(x0, x0, p[0]); p[1] = fmaf(x1, x1, p[1]); p[2] = fmaf(x2, x2, p[2]);
    p[3] = fmaf(x0, x1, p[3]); p[4] = fmaf(x0, x2, p[4]); p[5] = fmaf(x1, x2, p[5]);
    if (!nofit)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) df_add_prod(uh[3 * c + d], ul[3 * c + d], av[c], m[d]);
  }
  double c[6];
  block_sum_vecf<6>(p, c, s_red);
  if (threadIdx.x < 6) C6[threadIdx.x] = (float)c[threadIdx.x];
  if (!nofit) block_sum_df9(uh, ul, redu, ui);
  __syncthreads();
}

// Mode 0 candidates of one fit row (lists of row crow): the nseg segment
// lists merged into keys[] in ascending order of their bound and trimmed to
// those at or below tau (at least k+1); returns their count and sets *tau_out.
// Called by the whole block; keys holds next_pow2(2 Kp) entries.
__device__ int merge_row_cands(const uint64_t* __restrict__ cand, const int* __restrict__ cand_n, int crow, int nseg,
                               int segstride, int Kp, int k1, float rthr, uint64_t* keys, int* s_total,
                               float* tau_out) {
  if (threadIdx.x == 0) {
    int t = 0;
    for (int s = 0; s < nseg; ++s) t += cand_n[(int64_t)crow * nseg + s];
    *s_total = t;
  }
  __syncthreads();
  const int t = *s_total;
  // streaming merge: keys[0, Kp) holds the best K' so far (ascending), each
  // segment's list (ascending, at most K' keys, as every screen publishes
  // it) is placed after it reversed, behind +inf padding, so the buffer is
  // bitonic and one merge pass (log2 P2 barriers instead of a full sort's
  // log2 P2 (log2 P2 + 1) / 2) sorts it; shared memory stays O(K').
  const int P2 = next_pow2(2 * Kp);
  for (int x = threadIdx.x; x < P2; x += blockDim.x) keys[x] = MDS_KEY_INF;
  __syncthreads();
  for (int s = 0; s < nseg; ++s) {
    const int ns = min(cand_n[(int64_t)crow * nseg + s], Kp);
    if (ns == 0) continue;  // (uniform over the block)
    const uint64_t* src = cand + ((int64_t)crow * nseg + s) * segstride;
    const int tail = P2 - Kp;
    for (int x = threadIdx.x; x < tail; x += blockDim.x)
      keys[Kp + x] = (x >= tail - ns) ? src[tail - 1 - x] : MDS_KEY_INF;
    __syncthreads();
    for (int j = P2 >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint64_t a = keys[i], b = keys[ixj];
          if (a > b) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  int total = min(t, Kp);
  float tau = (t >= Kp) ? mds_key_value(keys[Kp - 1]) : __int_as_float(0x7f800000);
  // The screen's final shared threshold of the row: every pair it left out
  // has a bound at or above it (when it came from the (k+1)-th bound, the
  // lists may hold fewer than K' keys).
  tau = fminf(tau, rthr);
  // Candidates whose bound is above tau cannot enter the k+1 best once the
  // (k+1)-th exact value is at most tau, which the guard check requires:
  // recheck only those at or below it (at least k+1 of them, so that a
  // failed guard is still seen).
  int within = 0;
  for (int b0 = 0; b0 < total; b0 += blockDim.x) {
    const int x = b0 + threadIdx.x;
    within += __syncthreads_count(x < total && mds_key_value(keys[x]) <= tau);
  }
  *tau_out = tau;
  return max(within, min(total, k1));
}

// One block per fit row (rows[b] or b). mode 0: merge nseg candidate lists of
// K' keys, recheck, select k+1. mode 1: every reference is a candidate
// (exact row). mode 2 (full matrix): write every exact distance in reference
// order. Output: out_d/out_i rows of width `width` at row index grow.
__global__ void __launch_bounds__(RC_THREADS, 4)
k_recheck(const float* __restrict__ Af, const float* __restrict__ Ar, const float* __restrict__ mu,
          const float* __restrict__ Ur, int nrows,
          const int* __restrict__ rowlist, int Nr, int Ap, int natoms, int nofit, int mode,
          const uint64_t* __restrict__ cand, const int* __restrict__ cand_n, int nseg, int segstride, int Kp, int k,
          double* __restrict__ out_d, int* __restrict__ out_i, int* __restrict__ flagged, int* __restrict__ nflag,
          const float* __restrict__ rowthr, const float* __restrict__ recf, const float* __restrict__ recr,
          float guard, unsigned long long* __restrict__ audit, int cand_by_row) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* sa = reinterpret_cast<float*>(smem_raw);                 // [3*Ap] a_i
  float* sd = sa + 3 * Ap;                                        // [CHUNK]
  int* cj = reinterpret_cast<int*>(sd + RC_CHUNK);                // [CHUNK]
  uint64_t* keys = reinterpret_cast<uint64_t*>(cj + RC_CHUNK);    // merge buffer / top list
  __shared__ int s_total;
  __shared__ double s_red[32 * 6];
  __shared__ float C6[6];
  __shared__ __align__(16) float ssum[RC_CHUNK * 10];  // per candidate: D, Q[9] (float2 stores)
  __shared__ float ui[18];                              // the row's U as double-float pairs
  __shared__ float redu[(RC_THREADS / 32) * 18];

  int lr = blockIdx.x;
  if (lr >= nrows) return;
  int grow = rowlist ? rowlist[lr] : lr;
  const float* af = Af + (int64_t)grow * 3 * Ap;
  for (int e = threadIdx.x; e < 3 * Ap; e += blockDim.x) sa[e] = af[e];
  row_constants(af, mu, Ap, natoms, nofit, C6, ui, s_red, redu);
  const int k1 = k + 1;

  if (mode == 2) {
    __syncthreads();
    for (int base = 0; base < Nr; base += RC_CHUNK) {
      int nc = min(RC_CHUNK, Nr - base);
      for (int c = threadIdx.x; c < nc; c += blockDim.x) cj[c] = base + c;
      __syncthreads();
      recheck_chunk(sa, ui, C6, Ar, Ur, Ap, cj, nc, nofit, sd, ssum);
      for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        out_d[(int64_t)grow * Nr + base + c] = (double)sd[c] * 10.0;
        out_i[(int64_t)grow * Nr + base + c] = base + c;
      }
      __syncthreads();
    }
    return;
  }

  // Candidate list in keys[0..total): merged and trimmed to K' (mode 0) or
  // implicit 0..Nr-1 (mode 1).
  int total;
  float tau;
  if (mode == 0) {
    total = merge_row_cands(cand, cand_n, cand_by_row ? grow : lr, nseg, segstride, Kp, k1,
                            rowthr ? __ldcg(rowthr + grow) : __int_as_float(0x7f800000), keys, &s_total, &tau);
  } else {
    total = Nr;
    tau = __int_as_float(0x7f800000);
  }
  // top list of the k+1 best exact (value, index) keys, after the candidate
  // list region: candidate list needs Kp (mode 0) entries, top list 2*CHUNK+k1.
  uint64_t* top = keys + (mode == 0 ? max(Kp, 1) : 0);
  int TP2 = 1;
  while (TP2 < k1 + RC_CHUNK) TP2 <<= 1;
  for (int x = threadIdx.x; x < TP2; x += blockDim.x) top[x] = MDS_KEY_INF;
  __syncthreads();
  // Candidates come in ascending order of their lower bound; once the (k+1)-th
  // exact RMSD^2 is below the next candidate's bound and not above tau, no
  // later candidate (nor any excluded pair, whose bound is at least tau) can
  // enter the k+1 best.
  __shared__ int s_stop;
  bool stopped = false;
  int base = 0;
  const int first = min(RC_CHUNK, (k1 + 8 + 31) / 32 * 32);
  // Audit of the screen's lower bound: every rechecked candidate has both
  // its bound b (screen value minus the guard) and its exact RMSD^2, so the
  // screen error the guard must cover, (b + guard E - exact) / E with E =
  // |a_i|^2 + |a_j|^2, is measured on exactly the pairs near the row's
  // threshold. A bound above the exact value by more than the FP32
  // recheck's own error (RMSD^2 to ~1.7e-5 relative in the worst case seen;
  // 3e-5 is allowed) is a guard violation: the row is flagged and finished
  // by the wider FP32 screen or exactly, and the call reports it.
  const bool auditing = audit != nullptr && mode == 0;
  const float Ei = auditing ? __ldg(recf + (int64_t)grow * MDS_REC + 15) : 0.0f;
  float a_coef = 0.0f;
  int a_viol = 0;
  while (base < total) {
    int nc = min((mode == 0 && base == 0) ? first : RC_CHUNK, total - base);
    for (int c = threadIdx.x; c < nc; c += blockDim.x)
      cj[c] = (mode == 0) ? mds_key_index(keys[base + c]) : base + c;
    __syncthreads();
    recheck_chunk(sa, ui, C6, Ar, Ur, Ap, cj, nc, nofit, sd, ssum);
    if (auditing)
      for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const float b = mds_key_value(keys[base + c]);
        if (b > 0.0f) {  // (bounds clamped at zero carry no error information)
          const float r2 = sd[c] * sd[c];
          const float E = Ei + __ldg(recr + (int64_t)cj[c] * MDS_REC + 15);
          if (E > 0.0f) a_coef = fmaxf(a_coef, (b + guard * E - r2) / E);
          a_viol += (b > r2 * (1.0f + 3e-5f)) ? 1 : 0;
        }
      }
    // place the chunk after the current k1 best and re-sort
    for (int c = threadIdx.x; c < RC_CHUNK; c += blockDim.x)
      top[k1 + c] = (c < nc) ? mds_pack_key(sd[c], cj[c]) : MDS_KEY_INF;
    for (int x = k1 + RC_CHUNK + threadIdx.x; x < TP2; x += blockDim.x) top[x] = MDS_KEY_INF;
    __syncthreads();
    block_bitonic_sort(top, TP2);
    base += nc;
    if (mode == 0 && base < total) {
      if (threadIdx.x == 0) {
        double dk = (double)mds_key_value(top[k1 - 1]);
        double next = (double)mds_key_value(keys[base]);
        s_stop = (dk * dk * (1.0 + 1e-6) < next && dk * dk * (1.0 + 1e-6) <= (double)tau) ? 1 : 0;
      }
      __syncthreads();
      if (s_stop) {
        stopped = true;
        break;
      }
    }
  }
  int violated = 0;
  if (audit) {
    // one atomic per warp: candidates rechecked, violations, largest error
    const int lane = threadIdx.x & 31;
    const unsigned cb = __reduce_max_sync(0xffffffffu, __float_as_uint(fmaxf(a_coef, 0.0f)));
    const int vs = __reduce_add_sync(0xffffffffu, (unsigned)a_viol);
    if (lane == 0) {
      if (cb) atomicMax(audit + 2, (unsigned long long)cb);
      if (vs) atomicAdd(audit + 1, (unsigned long long)vs);
    }
    if (threadIdx.x == 0) atomicAdd(audit + 0, (unsigned long long)base);
    violated = __syncthreads_or(a_viol > 0);
  }
  // guard: the (k+1)-th exact RMSD^2 must not exceed the smallest lower bound
  // of every excluded pair, and no rechecked bound may exceed its exact value.
  if (threadIdx.x == 0) {
    double dk = (double)mds_key_value(top[k1 - 1]);
    if (mode == 0 && (violated || (!stopped && !(dk * dk * (1.0 + 1e-6) <= (double)tau)))) {
      int pos = atomicAdd(nflag, 1);
      flagged[pos] = grow;
      if (violated) atomicAdd(audit + 3, 1ull);
    }
  }
  for (int x = threadIdx.x; x < k; x += blockDim.x) {
    uint64_t key = top[x + 1];
    out_d[(int64_t)grow * k + x] = (double)mds_key_value(key) * 10.0;
    out_i[(int64_t)grow * k + x] = mds_key_index(key);
  }
}

size_t recheck_smem(int Ap, int Kp, int k, int mode) {
  int k1 = k + 1;
  int TP2 = 1;
  while (TP2 < k1 + RC_CHUNK) TP2 <<= 1;
  size_t merge = 0;
  if (mode == 0) {
    merge = (size_t)std::max(Kp, 1);
  }
  size_t keys = std::max(merge + TP2, (size_t)0);
  return sizeof(float) * (3 * Ap + RC_CHUNK) + sizeof(int) * RC_CHUNK + sizeof(uint64_t) * keys;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
namespace {

void jacobi3(double a[9], double d[3], double v[9]) {
  for (int i = 0; i < 9; ++i) v[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
    if (off < 1e-300) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = a[3 * p + q];
        if (apq == 0.0) continue;
        double theta = (a[3 * q + q] - a[3 * p + p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = a[3 * k + p], akq = a[3 * k + q];
          a[3 * k + p] = c * akp - s * akq;
          a[3 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[3 * p + k], aqk = a[3 * q + k];
          a[3 * p + k] = c * apk - s * aqk;
          a[3 * q + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = v[3 * k + p], vkq = v[3 * k + q];
          v[3 * k + p] = c * vkp - s * vkq;
          v[3 * k + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) d[i] = a[4 * i];
}

}  // namespace

// Template mu = first reference frame rotated into its principal axes (so
// that sum mu mu^T is diagonal and the antisymmetric parts the screen needs
// stay small).
int build_template(mds_ctx* ctx, const float* dY0, int Ap, int natoms, bool nofit,
                   std::vector<double>& mu, double M0[9]) {
  std::vector<float> y(3 * Ap);
  MDS_CUDA(ctx, cudaMemcpyAsync(y.data(), dY0, sizeof(float) * 3 * Ap, cudaMemcpyDeviceToHost, ctx->stream));
  MDS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double C[9] = {0};
  for (int a = 0; a < natoms; ++a)
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) C[3 * c + d] += (double)y[c * Ap + a] * y[d * Ap + a];
  double P[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, ev[3];
  if (!nofit) {
    double Cc[9];
    std::copy(C, C + 9, Cc);
    jacobi3(Cc, ev, P);
    double det = P[0] * (P[4] * P[8] - P[5] * P[7]) - P[1] * (P[3] * P[8] - P[5] * P[6]) +
                 P[2] * (P[3] * P[7] - P[4] * P[6]);
    if (det < 0)
      for (int i = 0; i < 3; ++i) P[3 * i] = -P[3 * i];
  }
  mu.assign(3 * Ap, 0.0);
  for (int a = 0; a < natoms; ++a)
    for (int d = 0; d < 3; ++d) {
      double s = 0;
      for (int c = 0; c < 3; ++c) s += (double)y[c * Ap + a] * P[3 * c + d];
      mu[d * Ap + a] = s;
    }
  for (int i = 0; i < 9; ++i) M0[i] = 0;
  for (int a = 0; a < natoms; ++a)
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) M0[3 * c + d] += mu[c * Ap + a] * mu[d * Ap + a];
  return MDS_OK;
}

int launch_recheck(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Af, const float* Ar, const float* mu,
                   const float* Ur, int nrows, const int* rowlist, int mode,
                   const uint64_t* cand, const int* cand_n, int nseg, int segstride, int Kp, int k,
                   double* out_d, int* out_i, int* flagged, int* nflag, const float* rowthr,
                   const RecheckAudit* audit, int cand_by_row) {
  size_t smem = recheck_smem(pl.Ap, Kp, k, mode);
  if (mode == 0) {
    // the streaming merge works on the best K' plus one segment's K'
    int P2 = next_pow2(2 * Kp);
    int TP2 = 1;
    while (TP2 < k + 1 + RC_CHUNK) TP2 <<= 1;
    size_t keys = std::max((size_t)P2, (size_t)Kp + TP2);
    smem = sizeof(float) * (3 * pl.Ap + RC_CHUNK) + sizeof(int) * RC_CHUNK + sizeof(uint64_t) * keys;
  }
  if (smem > 227 * 1024)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "recheck needs %zu bytes of shared memory (natoms/k too large)", smem);
  static bool attr_set = false;  // once: launches may also happen while a stream is captured
  static size_t limit = 0;
  MDS_TRY(mds_allow_dyn_smem(ctx, k_recheck, &attr_set, &limit));
  if (smem > limit) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "recheck shared memory %zu > %zu", smem, limit);
  if (nrows > 0) ctx->stats.launches++;
  if (nrows > 0)
    k_recheck<<<nrows, RC_THREADS, smem, ctx->stream>>>(Af, Ar, mu, Ur, nrows, rowlist, pl.nref, pl.Ap, pl.natoms,
                                                        pl.nofit, mode, cand, cand_n, nseg, segstride, Kp, k,
                                                        out_d, out_i, flagged, nflag, rowthr,
                                                        audit ? audit->recf : nullptr, audit ? audit->recr : nullptr,
                                                        audit ? audit->guard : 0.0f,
                                                        audit ? audit->counters : nullptr, cand_by_row);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// Launch wrappers used by the resident serving path (serve.cu).
int launch_center(mds_ctx* ctx, const float* draw, int n, int natoms, int Ap, const float* dmass,
                  const float* dswn, float tm, float* Y, double* E) {
  if (n <= 0) return MDS_OK;
  ctx->stats.launches++;
  k_center<<<n, 128, 0, ctx->stream>>>(draw, n, natoms, Ap, dmass, dswn, tm, Y, E);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// dst[t] = frame idx[t] of src (fl floats per frame); src may be page-locked
// host memory read through its device mapping.
__global__ void k_gather_raw(const float* __restrict__ src, const int* __restrict__ idx, int n, int fl,
                             float* __restrict__ dst) {
  const int t = blockIdx.x;
  if (t >= n) return;
  const float* a = src + (int64_t)idx[t] * fl;
  float* b = dst + (int64_t)t * fl;
  for (int e = threadIdx.x; e < fl; e += blockDim.x) b[e] = a[e];
}

int launch_prep(mds_ctx* ctx, const float* draw, int n, int natoms, int Ap, const float* dmass, const float* dswn,
                float tm, const float* dmu, const double* dM0, int nofit, float* A, float* R, float* Uhl, int* bad,
                int fbase) {
  if (n <= 0) return MDS_OK;
  ctx->stats.launches += nofit ? 2 : 3;
  k_prep_sums<<<n, 128, 0, ctx->stream>>>(draw, n, natoms, Ap, dmass, dswn, tm, dmu, nofit, R, bad, fbase);
  if (!nofit) k_prep_rot<<<(n + 127) / 128, 128, 0, ctx->stream>>>(n, dM0, R);
  k_prep_out<<<n, 128, 0, ctx->stream>>>(draw, n, natoms, Ap, dswn, dmu, dM0, nofit, A, R, Uhl);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

int choose_nseg_fp32(int nfit, int num_sms, int nref) {
  int nrt = (nfit + SC_TM - 1) / SC_TM, nct = (nref + SC_TN - 1) / SC_TN;
  int best = 1;
  double besteff = 0;
  for (int s = 1; s <= 8 && s <= nct; ++s) {
    double waves = (double)nrt * s / num_sms;
    double eff = waves / std::ceil(waves);
    if (eff > besteff + 0.02) {
      besteff = eff;
      best = s;
    }
    if (eff >= 0.95) break;
  }
  return best;
}

static int choose_nseg(int nrowtiles, int num_sms, int ncoltiles) {
  int best = 1;
  double besteff = 0;
  for (int s = 1; s <= 8 && s <= ncoltiles; ++s) {
    double waves = (double)nrowtiles * s / num_sms;
    double eff = waves / std::ceil(waves);
    if (eff > besteff + 0.02) {
      besteff = eff;
      best = s;
    }
    if (eff >= 0.95) break;
  }
  return best;
}

int knn_rms_run(mds_ctx* ctx, KnnRmsPlan& pl, const float* draw_ref, const float* draw_fit,
                const float* hmass, double* dout_d, int* dout_i) {
  const int Ap = pl.Ap, natoms = pl.natoms;
  mds_knn_stats& st = ctx->stats;
  cudaStream_t s = ctx->stream;
  // masses: sqrt(w/M) per atom, tm = float sum in file order (reset_x)
  std::vector<float> swn(Ap, 0.f);
  float tm = 0.f;
  double M = 0;
  for (int a = 0; a < natoms; ++a) {
    tm += hmass[a];
    M += hmass[a];
  }
  if (!(M > 0)) return mds_fail(ctx, MDS_ERR_ARG, "total mass must be positive");
  for (int a = 0; a < natoms; ++a) swn[a] = (float)std::sqrt((double)hmass[a] / M);
  DevBuf dmass, dswn;
  MDS_TRY(dmass.alloc(ctx, sizeof(float) * natoms));
  MDS_TRY(dswn.alloc(ctx, sizeof(float) * Ap));
  MDS_CUDA(ctx, cudaMemcpyAsync(dmass.p, hmass, sizeof(float) * natoms, cudaMemcpyHostToDevice, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(dswn.p, swn.data(), sizeof(float) * Ap, cudaMemcpyHostToDevice, s));

  const bool same = (draw_fit == nullptr);
  const int nref = pl.nref, nfit = same ? nref : pl.nfit;
  const size_t frame_bytes = sizeof(float) * 3 * (size_t)natoms;
  // frames still on the host: chunked uploads that the superposition below
  // consumes chunk by chunk
  std::vector<int> cb_ref{0, nref}, cb_fit{0, nfit};
  int nc_ref = 1, nc_fit = 1;
  // Staged preparation (a set screened against itself from host frames, on
  // the tensor-core screen with tile skipping): the row-tile pivots' frames
  // are copied first and prepared on their own, so that as each upload chunk
  // lands its frames are superposed, split into the screen's operands, and
  // bounded against every pivot (the pivot pass over its row tiles) while
  // later chunks are still in flight. The kernels and results are those of
  // the unstaged order; only the order of the work changes.
  // (page-locked host frames only: the pivots' frames are read through the
  // device mapping of that memory, and only such uploads overlap anyway)
  // Both ends of the frames must be page-locked host memory, mapped for the
  // device as one range, so that the gather kernel can read any frame.
  const float* hmap = nullptr;
  if (pl.href && nref > 0) {
    const size_t span = frame_bytes * (size_t)nref - 1;
    const char* first = reinterpret_cast<const char*>(pl.href);
    cudaPointerAttributes pa, pb;
    if (cudaPointerGetAttributes(&pa, first) == cudaSuccess && cudaPointerGetAttributes(&pb, first + span) == cudaSuccess &&
        pa.type == cudaMemoryTypeHost && pb.type == cudaMemoryTypeHost && pa.devicePointer &&
        static_cast<const char*>(pb.devicePointer) == static_cast<const char*>(pa.devicePointer) + span)
      hmap = static_cast<const float*>(pa.devicePointer);
    cudaGetLastError();
  }
  const bool staged = hmap && same && pl.prec != MDS_PREC_FP32 && !pl.screen_keys && !pl.noskip && !pl.full &&
                      !pl.prep_dev && (nref + TC_FR_N - 1) / TC_FR_N >= 4;
  TcPivots spv;
  DevBuf praw(ctx), gidx(ctx);
  if (staged) MDS_TRY(tc_pivots_begin(ctx, pl, spv, true));
  if (pl.href)
    MDS_TRY(mds_upload_chunked(ctx, const_cast<float*>(draw_ref), pl.href, nref, frame_bytes, 0, cb_ref, &nc_ref,
                               staged ? TC_FR_N : 1));
  if (staged) {
    // the pivots' frames, and frame 0 (the template's) after them, gathered
    // from the host frames while the chunks are in flight
    std::vector<int> gi(spv.hidx);
    gi.push_back(0);
    MDS_TRY(gidx.alloc(ctx, sizeof(int) * gi.size()));
    MDS_CUDA(ctx, cudaMemcpyAsync(gidx.p, gi.data(), sizeof(int) * gi.size(), cudaMemcpyHostToDevice, s));
    MDS_TRY(praw.alloc(ctx, frame_bytes * gi.size()));
    k_gather_raw<<<(int)gi.size(), 128, 0, s>>>(hmap, gidx.as<int>(), (int)gi.size(), 3 * natoms, praw.as<float>());
    MDS_CUDA(ctx, cudaGetLastError());
  }
  if (pl.hfit && !same)
    MDS_TRY(mds_upload_chunked(ctx, const_cast<float*>(draw_fit), pl.hfit, nfit, frame_bytes, MDS_MAX_CHUNKS,
                               cb_fit, &nc_fit));
  // the first reference frame, centred, defines the template
  DevBuf Y0(ctx), E0(ctx);
  MDS_TRY(Y0.alloc(ctx, sizeof(float) * 3 * Ap));
  MDS_TRY(E0.alloc(ctx, sizeof(double)));
  st.launches = staged ? 1 : 0;  // (the pivots' gather)
  st.launches++;
  if (pl.href && !staged) MDS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->chunk_ev[0], 0));
  k_center<<<1, 128, 0, s>>>(staged ? praw.as<float>() + (size_t)spv.nP * 3 * natoms : draw_ref, 1, natoms, Ap,
                             dmass.as<float>(), dswn.as<float>(), tm, Y0.as<float>(), E0.as<double>());
  MDS_CUDA(ctx, cudaGetLastError());

  const int k = pl.k;
  DevBuf flagged(ctx), nflag(ctx);
  MDS_TRY(flagged.alloc(ctx, sizeof(int) * (size_t)std::max(nfit, 1)));
  MDS_TRY(nflag.alloc(ctx, sizeof(int)));

  // template and superposition
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  std::vector<double> mu;
  double M0[9];
  MDS_TRY(build_template(ctx, Y0.as<float>(), Ap, natoms, pl.nofit != 0, mu, M0));
  DevBuf dmu(ctx), dM0(ctx), Ar(ctx), Rr(ctx), Af(ctx), Rf(ctx);
  std::vector<float> muf(mu.begin(), mu.end());
  MDS_TRY(dmu.alloc(ctx, sizeof(float) * 3 * Ap));
  MDS_TRY(dM0.alloc(ctx, sizeof(double) * 9));
  MDS_CUDA(ctx, cudaMemcpyAsync(dmu.p, muf.data(), sizeof(float) * 3 * Ap, cudaMemcpyHostToDevice, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(dM0.p, M0, sizeof(double) * 9, cudaMemcpyHostToDevice, s));
  MDS_TRY(Ar.alloc(ctx, sizeof(float) * 3 * Ap * (size_t)nref));
  MDS_TRY(Rr.alloc(ctx, sizeof(float) * MDS_REC * (size_t)nref));
  DevBuf Ur(ctx);  // the reference frames' U = sum a mu^T as double-float pairs (recheck)
  MDS_TRY(Ur.alloc(ctx, sizeof(float) * 18 * (size_t)nref));
  // frames with a non-finite coordinate (reference set, fit set): smallest
  // index, checked at the call's first synchronisation after the screen
  DevBuf badf(ctx);
  MDS_TRY(badf.alloc(ctx, 2 * sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(badf.p, 0x7f, 2 * sizeof(int), s));
  // superposition, one upload chunk at a time
  auto prep_chunks = [&](const float* draw, bool host, const std::vector<int>& cb, int nc, int ev0, float* A,
                         float* R, float* U, int* bad) -> int {
    for (int c = 0; c < nc; ++c) {
      if (host) MDS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->chunk_ev[ev0 + c], 0));
      const int f0 = cb[c], nf = cb[c + 1] - cb[c];
      MDS_TRY(launch_prep(ctx, draw + (size_t)f0 * 3 * natoms, nf, natoms, Ap, dmass.as<float>(), dswn.as<float>(),
                          tm, dmu.as<float>(), dM0.as<double>(), pl.nofit, A + (size_t)f0 * 3 * Ap,
                          R + (size_t)f0 * MDS_REC, U ? U + (size_t)f0 * 18 : nullptr, bad, f0));
    }
    return MDS_OK;
  };
  // error words of the tensor-core launches, read at the call's
  // synchronisation after the recheck: [0..1] the pivot pass, [2..3] the
  // screen, then two per staged chunk's pivot pass
  DevBuf tcerr(ctx);
  const int nerr = 4 + 2 * MDS_MAX_CHUNKS;
  MDS_TRY(tcerr.alloc(ctx, nerr * sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(tcerr.p, 0, nerr * sizeof(int), s));
  TcOperands tcr, tcf;
  DevBuf slb(ctx);  // staged: lower bounds from every frame to every pivot [nP][n]
  if (staged) {
    MDS_TRY(launch_prep(ctx, praw.as<float>(), spv.nP, natoms, Ap, dmass.as<float>(), dswn.as<float>(), tm,
                        dmu.as<float>(), dM0.as<double>(), pl.nofit, spv.A.as<float>(), spv.R.as<float>(), nullptr,
                        nullptr, 0));
    MDS_TRY(tc_pivots_operand(ctx, pl, spv));
    MDS_TRY(tc_alloc(ctx, pl, nref, tcr, 1));
    MDS_TRY(tc_alloc(ctx, pl, nref, tcr, 0));
    MDS_TRY(slb.alloc(ctx, sizeof(float) * (size_t)spv.nP * nref));
    for (int c = 0; c < nc_ref; ++c) {
      MDS_CUDA(ctx, cudaStreamWaitEvent(s, ctx->chunk_ev[c], 0));
      const int f0 = cb_ref[c], f1 = cb_ref[c + 1];
      MDS_TRY(launch_prep(ctx, draw_ref + (size_t)f0 * 3 * natoms, f1 - f0, natoms, Ap, dmass.as<float>(),
                          dswn.as<float>(), tm, dmu.as<float>(), dM0.as<double>(), pl.nofit,
                          Ar.as<float>() + (size_t)f0 * 3 * Ap, Rr.as<float>() + (size_t)f0 * MDS_REC,
                          pl.nofit ? nullptr : Ur.as<float>() + (size_t)f0 * 18, badf.as<int>(), f0));
      MDS_TRY(tc_prepare_range(ctx, pl, Ar.as<float>(), nref, tcr, 1, f0, f1));
      MDS_TRY(tc_prepare_range(ctx, pl, Ar.as<float>(), nref, tcr, 0, f0, f1));
      MDS_TRY(tc_pivots_radii(ctx, pl, Ar.as<float>(), spv, f0, f1));
      MDS_TRY(tc_skip_bounds(ctx, pl, tcr, Rr.as<float>(), nref, spv, slb.as<float>(), tcerr.as<int>() + 4 + 2 * c,
                             f0, f1));
    }
  } else {
    MDS_TRY(prep_chunks(draw_ref, pl.href != nullptr, cb_ref, nc_ref, 0, Ar.as<float>(), Rr.as<float>(),
                        pl.nofit ? nullptr : Ur.as<float>(), badf.as<int>()));
  }
  const float* Afp = Ar.as<float>();
  const float* Rfp = Rr.as<float>();
  if (!same) {
    MDS_TRY(Af.alloc(ctx, sizeof(float) * 3 * Ap * (size_t)nfit));
    MDS_TRY(Rf.alloc(ctx, sizeof(float) * MDS_REC * (size_t)nfit));
    MDS_TRY(prep_chunks(draw_fit, pl.hfit != nullptr, cb_fit, nc_fit, MDS_MAX_CHUNKS, Af.as<float>(),
                        Rf.as<float>(), nullptr, badf.as<int>() + 1));
    Afp = Af.as<float>();
    Rfp = Rf.as<float>();
  }
  if (pl.prep_dev) {
    MDS_CUDA(ctx, cudaMemcpyAsync(pl.prep_dev, Ar.p, sizeof(float) * 3 * Ap * (size_t)nref,
                                  cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(pl.prep_rec, Rr.p, sizeof(float) * MDS_REC * (size_t)nref,
                                  cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    return MDS_OK;
  }
  if (pl.full) {
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    MDS_TRY(launch_recheck(ctx, pl, Afp, Ar.as<float>(), dmu.as<float>(), Ur.as<float>(), nfit, nullptr, 2, nullptr, nullptr, 1, 1,
                           1, 0, dout_d, dout_i, flagged.as<int>(), nflag.as<int>()));
    MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    int hbad[2] = {0, 0};
    MDS_CUDA(ctx, cudaMemcpyAsync(hbad, badf.p, sizeof(hbad), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
    st.recheck_ms = ms;
    st.passes = 0;
    if (hbad[0] != 0x7f7f7f7f)
      return mds_fail(ctx, MDS_ERR_ARG, "reference frame %d has a non-finite coordinate", hbad[0]);
    if (hbad[1] != 0x7f7f7f7f)
      return mds_fail(ctx, MDS_ERR_ARG, "fit frame %d has a non-finite coordinate", hbad[1]);
    return MDS_OK;
  }
  // tensor-core operands (split hi/lo), when that screen is selected
  if (pl.prec != MDS_PREC_FP32 && !staged) {
    MDS_TRY(tc_prepare(ctx, pl, Ar.as<float>(), nref, tcr, 1));
    MDS_TRY(tc_prepare(ctx, pl, Afp, nfit, same ? tcr : tcf, 0));
  }

  // first pass
  int Kp = pl.kprime;
  int ncoltiles = (nref + 63) / 64;
  int nseg = choose_nseg((nfit + 31) / 32, ctx->num_sms, ncoltiles);
  if (pl.prec != MDS_PREC_FP32) {
    nseg = tc_choose_nseg(ctx, pl, nfit);
    // A set screened against itself skips most tiles and its items differ
    // widely in cost: smaller items (about 24 per SM; the row tile's own
    // segment is handed out first) keep the CTAs' finishing times together.
    if (same) {
      const int nrt = (nfit + 39) / 40, nct = (nref + 79) / 80;
      nseg = std::min(std::max(nseg, (24 * ctx->num_sms + nrt - 1) / nrt), std::min(8, nct));
    }
  }
  if (pl.screen_keys) nseg = 1;
  DevBuf cand(ctx), cand_n(ctx), rows(ctx);
  const int segstride = (pl.prec == MDS_PREC_FP32) ? Kp : tc_seg_stride();
  MDS_TRY(cand.alloc(ctx, sizeof(uint64_t) * (size_t)nfit * nseg * segstride));
  MDS_TRY(cand_n.alloc(ctx, sizeof(int) * (size_t)nfit * nseg));
  MDS_CUDA(ctx, cudaMemsetAsync(nflag.p, 0, sizeof(int), s));
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  DevBuf rowthr(ctx), nmax(ctx);  // shared row thresholds of the tensor-core screen, max |a_j|^2
  DevBuf ntiles(ctx);             // tiles the tensor-core screen computed
  unsigned long long ht = 0;      // (read back after the recheck)
  long long dense_pairs = 0;
  DevBuf f_lb(ctx), f_rowlo(ctx);
  TcPivots f_pv;
  if (pl.prec == MDS_PREC_FP32) {
    // shared row thresholds and the (k+1)-th rule; for a set screened
    // against itself, tile skipping with the row-tile pivots, whose bounds
    // come from a dense pass of this screen over the pivots
    Fp32ScreenExtra ex;
    const bool keys_only = pl.screen_keys != nullptr;
    if (!keys_only) {
      MDS_TRY(rowthr.alloc(ctx, sizeof(float) * std::max(nfit, 1)));
      MDS_CUDA(ctx, cudaMemsetAsync(rowthr.p, 0x7f, sizeof(float) * std::max(nfit, 1), s));
      MDS_TRY(nmax.alloc(ctx, sizeof(float)));
      MDS_TRY(tc_rec_nmax(ctx, Rr.as<float>(), nref, nmax.as<float>()));
      MDS_TRY(ntiles.alloc(ctx, sizeof(unsigned long long)));
      MDS_CUDA(ctx, cudaMemsetAsync(ntiles.p, 0, sizeof(unsigned long long), s));
      ex.rowthr = rowthr.as<float>();
      ex.nmax = nmax.as<float>();
      ex.k1 = k + 1;
      ex.ntiles = ntiles.as<unsigned long long>();
    }
    ex.diag = same ? 1 : 0;
    const bool skipping = !keys_only && !pl.noskip && same && (nref + TC_FR_N - 1) / TC_FR_N >= 4;
    st.screen_launches = 1;
    if (skipping) {
      MDS_TRY(tc_skip_pivots(ctx, pl, Ar.as<float>(), Rr.as<float>(), f_pv, true));
      MDS_TRY(f_lb.alloc(ctx, sizeof(float) * (size_t)f_pv.nP * nfit));
      Fp32ScreenExtra dx;
      dx.dense = f_lb.as<float>();
      KnnRmsPlan pp = pl;
      pp.nref = f_pv.nP;
      MDS_TRY(launch_screen_fp32(ctx, pp, Afp, f_pv.A.as<float>(), Rfp, f_pv.R.as<float>(), nfit, nullptr, 32,
                                 choose_nseg_fp32(nfit, ctx->num_sms, f_pv.nP), nullptr, nullptr, &dx));
      MDS_TRY(f_rowlo.alloc(ctx, sizeof(float) * (size_t)f_pv.nP * f_pv.nC));
      MDS_TRY(tc_skip_rowlo(ctx, f_pv, f_lb.as<float>(), nfit, f_rowlo.as<float>()));
      ex.pivlb = f_lb.as<float>();
      ex.prad = f_pv.rad.as<float>();
      ex.rowlo = f_rowlo.as<float>();
      ex.nR = f_pv.nP;
      ex.nC = f_pv.nC;
      ex.nfit = nfit;
      dense_pairs = (long long)f_pv.nP * nfit;
      st.screen_launches = 2;
    }
    MDS_TRY(launch_screen_fp32(ctx, pl, Afp, Ar.as<float>(), Rfp, Rr.as<float>(), nfit, nullptr, Kp, nseg,
                               cand.as<uint64_t>(), cand_n.as<int>(), &ex));
  } else {
    // tile skipping by the triangle inequality once there are tiles to skip
    // (a set screened against itself uses row-tile pivots)
    TcSkip sk;
    TcPivots upv;
    DevBuf ulb(ctx), rowlo(ctx), farw(ctx), farp(ctx);
    TcPivots& pv = staged ? spv : upv;  // (staged: pivots, radii and bounds made with the chunks)
    DevBuf& lb = staged ? slb : ulb;
    const bool skipping = !pl.screen_keys && !pl.noskip && (nref + 79) / 80 >= 4;
    if (skipping) {
      if (!staged) {
        MDS_TRY(tc_skip_pivots(ctx, pl, Ar.as<float>(), Rr.as<float>(), pv, same));
        MDS_TRY(lb.alloc(ctx, sizeof(float) * (size_t)pv.nP * nfit));
        MDS_TRY(tc_skip_bounds(ctx, pl, same ? tcr : tcf, Rfp, nfit, pv, lb.as<float>(), tcerr.as<int>()));
      }
      sk.pivlb = lb.as<float>();
      sk.prad = pv.rad.as<float>();
      if (same) {
        MDS_TRY(rowlo.alloc(ctx, sizeof(float) * (size_t)pv.nP * pv.nC));
        MDS_TRY(tc_skip_rowlo(ctx, pv, lb.as<float>(), nfit, rowlo.as<float>()));
        sk.rowlo = rowlo.as<float>();
        sk.piv2 = 1;
        if (nseg > 1) {
          const size_t nfar = (size_t)pv.nP * (nseg - 1);
          MDS_TRY(farw.alloc(ctx, sizeof(int) * (3 * 1024 + nfar)));
          MDS_TRY(farp.alloc(ctx, sizeof(int) * nfar));
          MDS_TRY(tc_far_order(ctx, pv, lb.as<float>(), rowlo.as<float>(), nfit, nseg, farw.as<int>(),
                               farp.as<int>()));
          sk.far_perm = farp.as<int>();
        }
      }
    }
    // (the candidate-screen diagnostic keeps plain K' lists: no (k+1)-th rule)
    MDS_TRY(rowthr.alloc(ctx, sizeof(float) * std::max(nfit, 1)));
    MDS_TRY(nmax.alloc(ctx, sizeof(float)));
    MDS_TRY(tc_rec_nmax(ctx, Rr.as<float>(), nref, nmax.as<float>()));
    MDS_TRY(ntiles.alloc(ctx, sizeof(unsigned long long)));
    MDS_CUDA(ctx, cudaMemsetAsync(ntiles.p, 0, sizeof(unsigned long long), s));
    MDS_TRY(launch_screen_tc(ctx, pl, same ? tcr : tcf, tcr, Rfp, Rr.as<float>(), nfit, Kp, nseg,
                             cand.as<uint64_t>(), cand_n.as<int>(), pl.screen_keys ? nullptr : tcerr.as<int>() + 2,
                             skipping ? &sk : nullptr, nullptr,
                             rowthr.as<float>(), pl.screen_keys ? nullptr : nmax.as<float>(),
                             ntiles.as<unsigned long long>()));
    st.screen_launches = skipping ? 2 : 1;
    // (staged: the pivot pass ran with the chunks, its time in the prep stage)
    dense_pairs = skipping ? (long long)pv.nP * nfit : 0;
  }
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  if (pl.screen_keys) {
    MDS_CUDA(ctx, cudaMemcpy2DAsync(pl.screen_keys, sizeof(uint64_t) * Kp, cand.p, sizeof(uint64_t) * segstride,
                                    sizeof(uint64_t) * Kp, nfit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(pl.screen_counts, cand_n.p, sizeof(int) * nfit, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    float t12 = 0;
    cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
    st.screen_ms = t12;
    st.kprime = Kp;
    return MDS_OK;
  }
  // the recheck audits the screen's bounds on the pairs it rechecks
  DevBuf audit_c(ctx);
  MDS_TRY(audit_c.alloc(ctx, 4 * sizeof(unsigned long long)));
  MDS_CUDA(ctx, cudaMemsetAsync(audit_c.p, 0, 4 * sizeof(unsigned long long), s));
  RecheckAudit audit;
  audit.recf = Rfp;
  audit.recr = Rr.as<float>();
  audit.guard = (pl.prec == MDS_PREC_FP32) ? pl.guard_fp32 : pl.guard_tc;
  audit.counters = audit_c.as<unsigned long long>();
  MDS_TRY(launch_recheck(ctx, pl, Afp, Ar.as<float>(), dmu.as<float>(), Ur.as<float>(), nfit, nullptr, 0,
                         cand.as<uint64_t>(), cand_n.as<int>(), nseg, segstride, Kp, k, dout_d, dout_i,
                         flagged.as<int>(), nflag.as<int>(), rowthr.p ? rowthr.as<float>() : nullptr, &audit));
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
  int hflag = 0, hbad[2] = {0, 0}, herr[4 + 2 * MDS_MAX_CHUNKS] = {};
  unsigned long long hc[4] = {0, 0, 0, 0};
  MDS_CUDA(ctx, cudaMemcpyAsync(herr, tcerr.p, sizeof(herr), cudaMemcpyDeviceToHost, s));
  if (ntiles.p) MDS_CUDA(ctx, cudaMemcpyAsync(&ht, ntiles.p, sizeof(ht), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(&hflag, nflag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(hc, audit_c.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(hbad, badf.p, sizeof(hbad), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  for (int c = 0; c < MDS_MAX_CHUNKS; ++c)
    if (herr[4 + 2 * c] && !herr[0]) herr[0] = herr[4 + 2 * c];
  if (herr[0] || herr[2])
    return mds_fail(ctx, MDS_ERR_TIMEOUT, "tensor-core screen: a bounded wait timed out (pass %s, role %d)",
                    herr[0] ? "pivots" : "screen", herr[0] ? herr[0] : herr[2]);
  // (every loop of the screen and recheck is bounded, so such frames only
  // make their own values meaningless; the call reports them as an error)
  if (hbad[0] != 0x7f7f7f7f)
    return mds_fail(ctx, MDS_ERR_ARG, "reference frame %d has a non-finite coordinate", hbad[0]);
  if (hbad[1] != 0x7f7f7f7f)
    return mds_fail(ctx, MDS_ERR_ARG, "fit frame %d has a non-finite coordinate", hbad[1]);
  st.recheck_pairs = (long long)hc[0];
  st.guard_violations = (int)hc[1];
  {
    const unsigned bits = (unsigned)hc[2];
    float f;
    std::memcpy(&f, &bits, sizeof(f));
    st.screen_err_max = f;
  }
  st.guard_coef = audit.guard;
  st.rows_audit_flagged = (int)hc[3];
  float t01 = 0, t12 = 0, t23 = 0;
  cudaEventElapsedTime(&t01, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
  cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
  st.prep_ms = t01;
  st.screen_ms = t12;
  st.recheck_ms = t23;
  st.kprime = Kp;
  st.rows_flagged = hflag;
  st.passes = 1;
  // (ht landed with the sync above)
  st.screen_pairs = (long long)ht * (pl.prec == MDS_PREC_FP32 ? 32 * 64 : TC_FR_M * TC_FR_N) + dense_pairs;

  // re-screen flagged rows with more candidates (FP32 screen), then exact rows
  while (hflag > 0) {
    std::vector<int> hrows(hflag);
    MDS_CUDA(ctx, cudaMemcpyAsync(hrows.data(), flagged.p, sizeof(int) * hflag, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    std::sort(hrows.begin(), hrows.end());
    MDS_TRY(rows.alloc(ctx, sizeof(int) * hflag));
    MDS_CUDA(ctx, cudaMemcpyAsync(rows.p, hrows.data(), sizeof(int) * hflag, cudaMemcpyHostToDevice, s));
    MDS_CUDA(ctx, cudaMemsetAsync(nflag.p, 0, sizeof(int), s));
    Kp = std::min(Kp * 4, 448);
    st.passes++;
    if (Kp >= nref || st.passes > 3) {
      // exact rows: every reference is a candidate
      MDS_TRY(launch_recheck(ctx, pl, Afp, Ar.as<float>(), dmu.as<float>(), Ur.as<float>(), hflag, rows.as<int>(), 1, nullptr,
                             nullptr, 1, 1, 1, k, dout_d, dout_i, flagged.as<int>(), nflag.as<int>()));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      break;
    }
    // few rows: spread each over many column segments so the whole GPU works
    const int nrt2 = (hflag + SC_TM - 1) / SC_TM;
    const int nseg2 = std::max(1, std::min((2 * ctx->num_sms + nrt2 - 1) / nrt2, (nref + SC_TN - 1) / SC_TN));
    MDS_TRY(cand.alloc(ctx, sizeof(uint64_t) * (size_t)hflag * nseg2 * Kp));
    MDS_TRY(cand_n.alloc(ctx, sizeof(int) * (size_t)hflag * nseg2));
    MDS_TRY(launch_screen_fp32(ctx, pl, Afp, Ar.as<float>(), Rfp, Rr.as<float>(), hflag, rows.as<int>(), Kp,
                               nseg2, cand.as<uint64_t>(), cand_n.as<int>()));
    RecheckAudit audit2 = audit;  // the re-screen's bounds carry the FP32 guard
    audit2.guard = pl.guard_fp32;
    MDS_TRY(launch_recheck(ctx, pl, Afp, Ar.as<float>(), dmu.as<float>(), Ur.as<float>(), hflag, rows.as<int>(), 0,
                           cand.as<uint64_t>(), cand_n.as<int>(), nseg2, Kp, Kp, k, dout_d, dout_i,
                           flagged.as<int>(), nflag.as<int>(), nullptr, &audit2));
    MDS_CUDA(ctx, cudaMemcpyAsync(&hflag, nflag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
  }
  return MDS_OK;
}
