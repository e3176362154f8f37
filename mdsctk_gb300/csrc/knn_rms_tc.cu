// knn_rms_tc.cu -- the all-pairs candidate screen of knn_rms on the 5th
// generation tensor cores (tcgen05 + TMEM + TMA), split precision.
//
// The nine A-long contractions of every frame pair (the 3x3 deviation Gram
// G_ij = sum_a a_i(a) a_j(a)^T) are one GEMM: rows (frame, xyz) of the fit
// set times rows (frame, xyz) of the reference set, reduced over atoms.
// Each operand is split x = hi + lo in BF16 (or FP16) and the product is
// hi*hi + hi*lo + lo*hi, accumulated in FP32 in TMEM.
//
// CTA tile: M = 128 TMEM lanes = 40 fit frames (each 32-lane quarter holds
// 10 frames x 3 coordinates, two padding lanes), N = 240 columns = 80
// reference frames stored coordinate-major (x of 80 frames, then y, then z).
// Reduction in K-blocks of 32 atoms through a 4-stage TMA pipeline
// (64-byte swizzle). Two TMEM accumulators (2 x 240 of 512 columns) let the
// MMA of one column tile run under the epilogue of the previous one.
//
// Warp roles (576 threads, one CTA per SM, persistent over work items =
// (row tile, column segment)):
//   warp 0       TMA producer (one thread)
//   warp 1       TMEM allocator + MMA issuer (one thread)
//   warps 2..17  epilogue: four warps per TMEM lane quarter, each taking a
//                quarter of the column chunks. A 3-lane shuffle transpose
//                gives each lane the full 3x3 Gram of one pair; the shifted
//                QCP bound (qcp.cuh) and the guard give the lower bound of
//                RMSD^2; passing pairs are appended to a per-(row, segment)
//                buffer of 512 keys in global memory, cut back to the best K'
//                by a warp radix select when it fills.
// Column tiles are visited outward from the row tile's own frames when a set
// is screened against itself, so thresholds tighten early.
// Every wait is bounded; on a timeout the kernel records an error, drains,
// frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "knn_common.cuh"
#include "qcp.cuh"
#include "tc_ptx.cuh"
#include "tc_select.cuh"

// TC_FR_M / TC_FR_N (frames per row / column tile) come from knn_common.cuh
#define TC_M 128
#define TC_N 240
#define TC_KB 32
#define TC_STAGES 4
#define TC_THREADS 576
#define TC_EPI_WARPS 16
// TC_CAPG (keys per list) comes from tc_select.cuh
#define TC_A_BYTES (TC_M * TC_KB * 2)
#define TC_B_BYTES (TC_N * TC_KB * 2)
#define TC_STAGE_BYTES (2 * TC_A_BYTES + 2 * TC_B_BYTES)
#define TC_TMEM_COLS 512
#define TC_SLACK 16  // keys beyond K' that trigger a compaction (K' + 16 + 80 <= TC_CAPG)

// ---------------------------------------------------------------------------
// operand preparation: FP32 deviations [n][3][Ap] -> split hi|lo rows
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T to_lp(float x);
template <>
__device__ __forceinline__ __nv_bfloat16 to_lp<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <>
__device__ __forceinline__ __half to_lp<__half>(float x) { return __float2half_rn(x); }
template <class T>
__device__ __forceinline__ float from_lp(T x);
template <>
__device__ __forceinline__ float from_lp<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }
template <>
__device__ __forceinline__ float from_lp<__half>(__half x) { return __half2float(x); }

// layout 0 (fit side, A): row t*128 + q*32 + 3f + c  <- frame t*40 + q*10 + f
// layout 1 (ref side, B): row t*240 + c*80 + g        <- frame t*80 + g
// One thread per 8 consecutive atoms of a row: two 16-byte loads, two
// 16-byte stores (hi, lo).
template <class T>
__device__ __forceinline__ unsigned short lp_bits(T x);
template <>
__device__ __forceinline__ unsigned short lp_bits<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat16_as_ushort(x); }
template <>
__device__ __forceinline__ unsigned short lp_bits<__half>(__half x) { return __half_as_ushort(x); }

template <class T>
__global__ void k_tc_split(const float* __restrict__ dev, int n, int Ap, int layout, int r0, int rows, float scale,
                           T* __restrict__ out) {
  // operand rows [r0, rows)
  const int A8 = Ap >> 3;
  const int64_t idx = (int64_t)r0 * A8 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)rows * A8) return;
  const int r = (int)(idx / A8), k = (int)(idx % A8) * 8;
  int frame, c;
  bool valid;
  if (layout == 0) {
    const int t = r / TC_M, w = r % TC_M, q = w / 32, l = w % 32;
    frame = t * TC_FR_M + q * 10 + l / 3;
    c = l % 3;
    valid = (l < 30) && frame < n;
  } else {
    const int t = r / TC_N, w = r % TC_N;
    c = w / TC_FR_N;
    frame = t * TC_FR_N + w % TC_FR_N;
    valid = frame < n;
  }
  float x[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (valid) {
    const float4* src = reinterpret_cast<const float4*>(dev + ((int64_t)frame * 3 + c) * Ap + k);
    const float4 a = __ldg(src), b = __ldg(src + 1);
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
  }
  unsigned short hb[8], lb[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const float v = x[e] * scale;
    const T hi = to_lp<T>(v);
    hb[e] = lp_bits<T>(hi);
    lb[e] = lp_bits<T>(to_lp<T>(v - from_lp<T>(hi)));
  }
  uint4 h4, l4;
  h4.x = hb[0] | ((unsigned)hb[1] << 16); h4.y = hb[2] | ((unsigned)hb[3] << 16);
  h4.z = hb[4] | ((unsigned)hb[5] << 16); h4.w = hb[6] | ((unsigned)hb[7] << 16);
  l4.x = lb[0] | ((unsigned)lb[1] << 16); l4.y = lb[2] | ((unsigned)lb[3] << 16);
  l4.z = lb[4] | ((unsigned)lb[5] << 16); l4.w = lb[6] | ((unsigned)lb[7] << 16);
  *reinterpret_cast<uint4*>(out + (int64_t)r * 2 * Ap + k) = h4;
  *reinterpret_cast<uint4*>(out + (int64_t)r * 2 * Ap + Ap + k) = l4;
}

static float tc_scale(unsigned prec) { return prec == MDS_PREC_FP16X3 ? 64.0f : 1.0f; }

static int tc_layout_rows(int n, int layout) {
  return (layout == 0) ? (n + TC_FR_M - 1) / TC_FR_M * TC_M : (n + TC_FR_N - 1) / TC_FR_N * TC_N;
}

int tc_alloc(mds_ctx* ctx, const KnnRmsPlan& pl, int n, TcOperands& op, int layout) {
  const int rows = tc_layout_rows(n, layout);
  DevBuf& buf = (layout == 0) ? op.A : op.B;
  MDS_TRY(buf.alloc(ctx, (size_t)rows * 2 * pl.Ap * 2));
  if (layout == 0) op.rowsA = rows; else op.rowsB = rows;
  op.n = n;
  op.K = pl.Ap;
  return MDS_OK;
}

int tc_prepare_range(mds_ctx* ctx, const KnnRmsPlan& pl, const float* dev, int n, TcOperands& op, int layout,
                     int f0, int f1) {
  if (f0 % TC_FR_N || (f1 < n && f1 % TC_FR_N))
    return mds_fail(ctx, MDS_ERR_INTERNAL, "operand range [%d, %d) not aligned to %d frames", f0, f1, TC_FR_N);
  // a row tile of layout 0 holds TC_FR_M frames in TC_M rows, a column tile
  // of layout 1 TC_FR_N frames in TC_N rows
  const int r0 = (layout == 0) ? f0 / TC_FR_M * TC_M : f0 / TC_FR_N * TC_N;
  const int r1 = tc_layout_rows(f1, layout);
  if (r1 <= r0) return MDS_OK;
  DevBuf& buf = (layout == 0) ? op.A : op.B;
  const int64_t total = (int64_t)(r1 - r0) * (pl.Ap / 8);
  const int blocks = (int)((total + 255) / 256);
  ctx->stats.launches++;
  if (pl.prec == MDS_PREC_FP16X3)
    k_tc_split<__half><<<blocks, 256, 0, ctx->stream>>>(dev, n, pl.Ap, layout, r0, r1, tc_scale(pl.prec),
                                                        buf.as<__half>());
  else
    k_tc_split<__nv_bfloat16><<<blocks, 256, 0, ctx->stream>>>(dev, n, pl.Ap, layout, r0, r1, tc_scale(pl.prec),
                                                               buf.as<__nv_bfloat16>());
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

int tc_prepare(mds_ctx* ctx, const KnnRmsPlan& pl, const float* dev, int n, TcOperands& op, int layout) {
  MDS_TRY(tc_alloc(ctx, pl, n, op, layout));
  return tc_prepare_range(ctx, pl, dev, n, op, layout, 0, n);
}

// ---------------------------------------------------------------------------
// the screen kernel
// ---------------------------------------------------------------------------
#define TC_TQ 8  // depth of the task ring (producer -> MMA thread and epilogue warps)
struct TcShared {
  uint64_t full[TC_STAGES], empty[TC_STAGES], tfull[2], tempty[2], done;
  uint64_t tq_full[TC_TQ], tq_empty[TC_TQ];
  int2 task[TC_TQ];  // (item, column tile); tile -1 ends an item, item -1 the stream
  int thr_item;      // the item whose rows' thresholds thr[] holds (-1: none)
  uint32_t tmem_base;
  int abortf;
  int cnt[TC_FR_M];
  float thr[TC_FR_M];
  float colrec[TC_FR_N * MDS_REC];  // records of the current column tile
  float rowrec[TC_FR_M * MDS_REC];  // records of the current row tile
  float gthr[TC_FR_M];              // rows' global thresholds, refreshed per tile
};

// per-warp shared scratch: the radix-select histogram, and the final sort of a
// row's list when it holds at most TC_SCR keys
#define TC_SCR 256
#define TC_SMEM_BYTES (TC_STAGES * TC_STAGE_BYTES + sizeof(TcShared) + TC_EPI_WARPS * TC_SCR * 8 + 1024)
static_assert(TC_SMEM_BYTES <= 227 * 1024, "screen shared memory exceeds the per-block limit");

__device__ __forceinline__ float sel3(int i, float a0, float a1, float a2) {
  return i == 0 ? a0 : (i == 1 ? a1 : a2);
}


// Column tiles of a segment [t0, t1) in the order the screen visits them:
// outward from tile td (td, td+1, td-1, td+2, ...). For a frame set screened
// against itself td is the tile holding the row tile's own frames, so a
// row's threshold becomes tight early (trajectory neighbours are close in
// time) and few later pairs pass it; otherwise td = t0 (plain order).
__device__ __forceinline__ int tile_order(int i, int t0, int t1, int td) {
  const int L = td - t0, Rn = t1 - 1 - td, m = min(L, Rn);
  if (i == 0) return td;
  if (i <= 2 * m) return (i & 1) ? td + (i + 1) / 2 : td - i / 2;
  const int j = i - 2 * m;
  return (Rn > L) ? td + m + j : td - m - j;
}

// Column segment holding the column tile of row tile rt's middle frame.
__device__ __forceinline__ int diag_seg(int rt, int nseg, int nct) {
  const int dt = min((rt * TC_FR_M + TC_FR_M / 2) / TC_FR_N, nct - 1);
  int s = 0;
  while (s + 1 < nseg && (int)((int64_t)nct * (s + 1) / nseg) <= dt) ++s;
  return s;
}

// Work item -> (row tile, column segment). A set screened against itself
// (diag) first hands out, row tile by row tile, the segment holding the row
// tile's own frames, and only then the other segments: by the time those
// start, the near tiles have set the shared row thresholds they skip by.
// The other segments come in the order far_perm gives (when not null: the
// estimated heaviest first, so that the longest items do not start last).
__device__ __forceinline__ void item_split(int item, int nrt, int nseg, int nct, int diag, const int* far_perm,
                                           int& rt, int& seg) {
  if (!diag || nseg == 1) {
    rt = item / nseg;
    seg = item % nseg;
    return;
  }
  if (item < nrt) {
    rt = item;
    seg = diag_seg(rt, nseg, nct);
    return;
  }
  const int k = far_perm ? __ldg(far_perm + (item - nrt)) : item - nrt;
  rt = k / (nseg - 1);
  const int s = k % (nseg - 1), sd = diag_seg(rt, nseg, nct);
  seg = s < sd ? s : s + 1;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
k_screen_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
            const float* __restrict__ recf, const float* __restrict__ recr, int nfit, int Nr, int Ap,
            int nofit, float guard, float ginv, uint32_t idesc, int Kp, int nseg, int nitems, int rt0, int diag,
            const float* __restrict__ pivlb, const float* __restrict__ prad, const float* __restrict__ rowlo,
            int piv2, const int* __restrict__ far_perm,
            float* __restrict__ dense, float* __restrict__ rowthr, const float* __restrict__ nmax, int k1,
            unsigned long long* __restrict__ ntiles,
            uint64_t* __restrict__ candbuf, int* __restrict__ cand_n, int* __restrict__ err, int stall) {
  // err[0]: error code; err[1]: next unclaimed work item (zeroed by the host).
  // Work items (row tile, column segment) are claimed dynamically by each
  // CTA's producer, which also decides which column tiles of the item to
  // compute and passes (item, tile) tasks in order to the MMA thread and the
  // epilogue warps through the task ring.
  //
  // Tile skipping (pivlb != null): RMSD is a metric, so for row i and any
  // frame j of column tile T with pivot p_T, RMSD(i, j) >= RMSD(i, p_T) -
  // RMSD(j, p_T) >= pivlb[T][i] - prad[T] = L. When every row of the row tile
  // has L > 0 and L^2 above its current threshold (the K'-th smallest bound
  // of its list, which only decreases), no pair of the tile can enter the
  // lists, and every such pair's true RMSD^2 exceeds the final threshold the
  // recheck verifies against -- the tile is not computed.
  // With row-tile pivots (piv2, a set screened against itself): pivot R is
  // the middle frame of row tile R and pivlb[R][i] bounds RMSD(i, p_R); column
  // tile T holds row tiles 2T and 2T+1, and prad[2T], prad[2T+1] bound the
  // distances of its frames to their pivots, so L is the larger of the two
  // pivots' bounds. Row tile R also has RMSD(i, p_R) <= r_R for its frames i,
  // so RMSD(i, j) >= RMSD(j, p_R) - r_R >= rowlo[R][T] = min over j in T of
  // the lower bound of RMSD(j, p_R), minus r_R. L is the largest of these.
  //
  // Row thresholds across segments (rowthr != null): each compaction lowers
  // rowthr[row] to its segment's K'-th bound (atomicMin). Every segment then
  // appends only below min(own threshold, rowthr), and the skip test uses it:
  // a segment holding K' keys below rowthr exists, so the recheck's final
  // threshold is at most rowthr and every pair left out lies above it.
  //
  // Thresholds from the (k+1)-th bound (nmax != null: the largest |a_j|^2 of
  // the reference set): a bound b is the screen value minus the guard
  // g (|a_i|^2 + |a_j|^2), and the screen value is within the guard of the
  // exact RMSD^2, so the exact value is at most b + 2g (|a_i|^2 + |a_j|^2).
  // With k+1 keys of a list at or below b_(k+1), the (k+1)-th exact RMSD^2 of
  // the row is at most b_(k+1) + 2g (|a_i|^2 + nmax) = t': no pair whose
  // bound is above t' can be among the k+1 best, so a compaction sets the
  // row threshold to min(K'-th bound, t'). The recheck verifies the (k+1)-th
  // exact value against the final shared threshold, as against the K'-th.
  //
  // Dense mode (dense != null; the pivot pass): every pair's lower bound of
  // RMSD (sqrt of the screen value) is written to dense[j][i]; no lists.
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* stages = base;
  TcShared* S = reinterpret_cast<TcShared*>(base + TC_STAGES * TC_STAGE_BYTES);
  uint64_t* scratch_all = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(S) + sizeof(TcShared));

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = Ap / TC_KB;
  const int ncoltiles = (Nr + TC_FR_N - 1) / TC_FR_N;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&S->full[s], 1);
      mbar_init(&S->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&S->tfull[b], 1);
      mbar_init(&S->tempty[b], TC_EPI_WARPS);
    }
    mbar_init(&S->done, 1);
    for (int i = 0; i < TC_TQ; ++i) {
      mbar_init(&S->tq_full[i], 1);
      mbar_init(&S->tq_empty[i], 1 + TC_EPI_WARPS);
    }
    S->abortf = 0;
    S->thr_item = -1;
    mbar_fence_init();
  }
  if (warp == 1) {
    tmem_alloc(&S->tmem_base, TC_TMEM_COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S->tmem_base;
  volatile int* abortf = &S->abortf;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // The whole warp runs the loop (the skip test uses every lane); lane 0
    // claims items, pushes tasks and issues the TMA loads.
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
    }
    uint32_t stage = 0, phase = 0, qs = 0;
    bool ok = true;
    // push one task; false if the wait timed out or the kernel aborts
    auto push = [&](int item, int tile) -> bool {
      const uint32_t slot = qs % TC_TQ, ph = (qs / TC_TQ) & 1;
      int good = 1;
      if (lane == 0) {
        good = mbar_wait(&S->tq_empty[slot], ph ^ 1, abortf, 1000000000ull, 1024) ? 1 : 0;
        if (good) {
          S->task[slot] = make_int2(item, tile);
          mbar_arrive(&S->tq_full[slot]);
        }
      }
      ++qs;
      return __shfl_sync(0xffffffffu, good, 0) != 0;
    };
    while (ok) {
      int item = 0;
      if (lane == 0) {
        item = atomicAdd(err + 1, 1);
        if (item >= nitems) item = -1;
      }
      item = __shfl_sync(0xffffffffu, item, 0);
      if (item < 0) {
        // (stall: an injected fault for the failure-path tests -- the end
        // marker is withheld, every load issued has been consumed, and the
        // other roles' bounded waits run out)
        if (!stall) ok = push(-1, -1);
        break;
      }
      int rt, seg;
      item_split(item, nitems / nseg, nseg, ncoltiles, diag, far_perm, rt, seg);
      rt += rt0;
      const int t0 = (int)((int64_t)ncoltiles * seg / nseg), t1 = (int)((int64_t)ncoltiles * (seg + 1) / nseg);
      const int td = diag ? min(max((rt * TC_FR_M + TC_FR_M / 2) / TC_FR_N, t0), t1 - 1) : t0;
      uint32_t skipbits = 0;  // bit b: tile tbase + b of the current batch of 8 is skipped
      int tbase = 0, test_at = 0;
      for (int ti = 0; ti < t1 - t0 && ok; ++ti) {
        const int tile = tile_order(ti, t0, t1, td);
        if (pivlb && ti == test_at) {
          // skip test of the next 8 tiles at once (4 lanes per tile, 10 rows
          // per lane: one round of loads instead of one per tile), against
          // the rows' thresholds now, which only tighten later. While some
          // row has no threshold yet (an item's first tiles), the test is
          // repeated at every tile, so tiles are skipped as soon as the first
          // thresholds arrive.
          // Before the epilogue has loaded this item's list thresholds
          // (S->thr still holds the previous item's rows), the shared row
          // thresholds alone are used: each is itself a valid threshold.
          skipbits = 0;
          tbase = ti;
          test_at = ti + 1;
          int live = (lane == 0) ? (*(volatile int*)&S->thr_item == item) : 0;
          live = __shfl_sync(0xffffffffu, live, 0);
          if (live || rowthr) {
            __threadfence_block();
            const int tj = ti + (lane >> 2), r0 = (lane & 3) * 10;
            bool can = tj < t1 - t0, open = false;
            if (can) {
              const int tb = tile_order(tj, t0, t1, td);
              const int pa = piv2 ? 2 * tb : tb;
              const bool pb = piv2 && 2 * tb + 1 < (nfit + TC_FR_M - 1) / TC_FR_M;
              const float rada = __ldg(prad + pa), radb = pb ? __ldg(prad + pa + 1) : 0.0f;
              const float Lrow = rowlo ? __ldg(rowlo + (int64_t)rt * ncoltiles + tb) : 0.0f;
#pragma unroll
              for (int x = 0; x < 10; ++x) {
                const int gi = rt * TC_FR_M + r0 + x;
                if (gi < nfit) {
                  float thr = live ? *(volatile float*)&S->thr[r0 + x] : INFINITY;
                  if (rowthr) thr = fminf(thr, __ldcg(rowthr + gi));
                  open |= !(thr < 1e30f);
                  float L = fmaxf(__ldg(pivlb + (int64_t)pa * nfit + gi) - rada, Lrow);
                  if (pb) L = fmaxf(L, __ldg(pivlb + (int64_t)(pa + 1) * nfit + gi) - radb);
                  if (!(L > 0.0f && L * L > thr)) can = false;
                }
              }
            }
            const unsigned bal = __ballot_sync(0xffffffffu, can);
            if (!__any_sync(0xffffffffu, open)) test_at = ti + 8;
            int still = 1;
            if (live) {  // the list thresholds read belong to this item: not moved on meanwhile
              still = (lane == 0) ? (*(volatile int*)&S->thr_item == item) : 0;
              still = __shfl_sync(0xffffffffu, still, 0);
            }
            if (still)
              for (int b = 0; b < 8; ++b)
                if (((bal >> (4 * b)) & 0xFu) == 0xFu) skipbits |= 1u << b;
          }
        }
        if ((skipbits >> (ti - tbase)) & 1u) continue;
        if (!(ok = push(item, tile))) break;
        if (lane == 0) {
          for (int kb = 0; kb < nkb; ++kb) {
            if (!mbar_wait(&S->empty[stage], phase ^ 1, abortf, 1000000000ull, 1024)) { ok = false; break; }
            unsigned char* st = stages + stage * TC_STAGE_BYTES;
            mbar_expect_tx(&S->full[stage], TC_STAGE_BYTES);
            tma_load_2d(st, &tmA, &S->full[stage], kb * TC_KB, rt * TC_M);
            tma_load_2d(st + TC_A_BYTES, &tmA, &S->full[stage], Ap + kb * TC_KB, rt * TC_M);
            tma_load_2d(st + 2 * TC_A_BYTES, &tmB, &S->full[stage], kb * TC_KB, tile * TC_N);
            tma_load_2d(st + 2 * TC_A_BYTES + TC_B_BYTES, &tmB, &S->full[stage], Ap + kb * TC_KB, tile * TC_N);
            if (++stage == TC_STAGES) { stage = 0; phase ^= 1; }
          }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      }
      if (ok) ok = push(item, -1);
    }
    if (!ok && lane == 0) {
      atomicMax(err, 1);
      *abortf = 1;
      // drain: every issued stage completes or times out
      for (int s = 0; s < TC_STAGES; ++s) {
        volatile int dummy = 0;
        mbar_wait(&S->full[s], 0, &dummy, 50000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      uint32_t stage = 0, phase = 0, acc = 0;
      bool ok = true;
      const uint32_t sbase = smem_u32(stages);
      for (uint32_t qs = 0; ok; ++qs) {
        const uint32_t slot = qs % TC_TQ, qph = (qs / TC_TQ) & 1;
        if (!mbar_wait(&S->tq_full[slot], qph, abortf, 1000000000ull, 64)) { ok = false; break; }
        const volatile int* tv = reinterpret_cast<volatile int*>(&S->task[slot]);
        const int2 t = make_int2(tv[0], tv[1]);
        mbar_arrive(&S->tq_empty[slot]);
        if (t.x < 0) break;
        if (t.y < 0) continue;
        const uint32_t b = acc & 1, aph = (acc >> 1) & 1;
        if (!mbar_wait(&S->tempty[b], aph ^ 1, abortf, 1000000000ull, 64)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tbase + b * 256;
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&S->full[stage], phase, abortf, 1000000000ull, 64)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = sbase + stage * TC_STAGE_BYTES;
#pragma unroll
          for (int ks = 0; ks < TC_KB / 16; ++ks) {
            const uint64_t ahi = umma_desc_sw64(st + ks * 32);
            const uint64_t alo = umma_desc_sw64(st + TC_A_BYTES + ks * 32);
            const uint64_t bhi = umma_desc_sw64(st + 2 * TC_A_BYTES + ks * 32);
            const uint64_t blo = umma_desc_sw64(st + 2 * TC_A_BYTES + TC_B_BYTES + ks * 32);
            umma_f16(d, ahi, bhi, idesc, (kb | ks) != 0);
            umma_f16(d, ahi, blo, idesc, 1);
            umma_f16(d, alo, bhi, idesc, 1);
          }
          umma_commit(&S->empty[stage]);
          if (++stage == TC_STAGES) { stage = 0; phase ^= 1; }
        }
        if (ok) umma_commit(&S->tfull[b]);
        ++acc;
      }
      if (!ok) {
        atomicMax(err, 2);
        *abortf = 1;
      }
      if (ntiles && acc) atomicAdd(ntiles, (unsigned long long)acc);  // tiles computed
      // all MMAs of this thread retire before TMEM is freed
      umma_commit(&S->done);
      volatile int dummy = 0;
      mbar_wait(&S->done, 0, &dummy, 200000000ull);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;
    const int q = warp & 3;          // TMEM lane quarter of this warp
    const int h = ew >> 2;           // column quarter: chunks [ci0, ci1) of the 10
    const int ci0 = (h * 10) / 4, ci1 = ((h + 1) * 10) / 4;
    const int f = lane / 3, c = lane % 3;
    const int rloc = q * 10 + f;     // row within the 40-frame tile (f < 10)
    uint64_t* scratch = scratch_all + ew * TC_SCR;
    const float INF = __int_as_float(0x7f800000);
    const float* rrec = S->rowrec + min(rloc, TC_FR_M - 1) * MDS_REC;  // lanes 30, 31 (f = 10) are padding
    uint32_t acc = 0;
    bool ok = true;
    int cur = -1, rt = 0, seg = 0, grow = 0, ntile = 0;
    bool rowok = false;
    // The epilogue warps meet at named barrier 1 three times per tile: after
    // the task read (every warp has finished the previous tile, its
    // compactions and any publishing), after the accumulator is ready, and
    // after the pairs are appended (before compaction). A failed bounded
    // wait is ANDed into the first two, so all warps leave together.
    for (uint32_t qs = 0;; ++qs) {
      const uint32_t slot = qs % TC_TQ, qph = (qs / TC_TQ) & 1;
      const bool got = mbar_wait(&S->tq_full[slot], qph, abortf);
      int2 task = make_int2(-1, -1);
      if (got) {
        const volatile int* tv = reinterpret_cast<volatile int*>(&S->task[slot]);
        task = make_int2(tv[0], tv[1]);
      }
      __syncwarp();
      if (!bar_and(1, TC_EPI_WARPS * 32, got)) { ok = false; break; }
      if (lane == 0) mbar_arrive(&S->tq_empty[slot]);
      if (task.x < 0) break;
      if (task.x != cur) {
        // start of an item: row records and this warp's rows' lists
        cur = task.x;
        item_split(cur, nitems / nseg, nseg, ncoltiles, diag, far_perm, rt, seg);
        rt += rt0;
        grow = rt * TC_FR_M + rloc;
        rowok = (f < 10) && grow < nfit;
        ntile = 0;
        for (int e = ew * 32 + lane; e < TC_FR_M * MDS_REC; e += TC_EPI_WARPS * 32) {
          const int r = rt * TC_FR_M + e / MDS_REC;
          S->rowrec[e] = (r < nfit) ? __ldg(recf + (int64_t)r * MDS_REC + e % MDS_REC) : 0.f;
        }
        if (lane < 3 && h + 4 * lane < 10) {
          const int fr = h + 4 * lane;
          S->cnt[q * 10 + fr] = 0;
          S->thr[q * 10 + fr] = INF;
        }
      }
      if (task.y < 0) {
        // end of the item: sort and publish this warp's rows (their appends
        // and compactions are complete; the next task's barrier separates
        // this from the next item's resets)
        if (!dense)
          for (int fr = h; fr < 10; fr += 4) {
            const int r = q * 10 + fr;
            const int gr = rt * TC_FR_M + r;
            if (gr >= nfit) continue;
            int n = min(S->cnt[r], TC_CAPG);
            uint64_t* src = candbuf + ((int64_t)gr * nseg + seg) * TC_CAPG;
            // keys above the row's threshold now (appended under a looser
            // one) are dropped: the recheck's threshold is at most this one
            const float tp = fminf(S->thr[r], rowthr ? __ldcg(rowthr + gr) : INF);
            if (tp < INF) {
              int m = 0;
              for (int x0 = 0; x0 < n; x0 += 32) {
                const int x = x0 + lane;
                const uint64_t key = (x < n) ? src[x] : MDS_KEY_INF;
                const bool keep = x < n && mds_key_value(key) <= tp;
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) src[m + __popc(bal & ((1u << lane) - 1u))] = key;  // at or below the lane's own slot
                m += __popc(bal);
                __syncwarp();
              }
              n = m;
            }
            if (n > Kp) {
              warp_select_keep(src, n, Kp, reinterpret_cast<int*>(scratch), lane);
              n = Kp;
            }
            int P2 = 32;
            while (P2 < n) P2 <<= 1;
            if (n <= 1) {
            } else if (P2 <= TC_SCR) {
              for (int x = lane; x < n; x += 32) scratch[x] = src[x];
              __syncwarp();
              warp_bitonic_sort(scratch, n, P2, lane);
              for (int x = lane; x < n; x += 32) src[x] = scratch[x];
            } else {
              warp_bitonic_sort(src, n, TC_CAPG, lane);  // in place (global; __syncwarp orders it)
            }
            if (lane == 0) cand_n[(int64_t)gr * nseg + seg] = n;
            __syncwarp();
          }
        continue;
      }
      const int tile = task.y;
      const uint32_t b = acc & 1, aph = (acc >> 1) & 1;
      // column records of this tile (the previous tile's readers passed the
      // task barrier)
      for (int e = ew * 32 + lane; e < TC_FR_N * MDS_REC; e += TC_EPI_WARPS * 32) {
        const int j = tile * TC_FR_N + e / MDS_REC;
        S->colrec[e] = (j < Nr) ? __ldg(recr + (int64_t)j * MDS_REC + e % MDS_REC) : 0.f;
      }
      if (ew == 0)
        for (int r = lane; r < TC_FR_M; r += 32) {
          const int gi = rt * TC_FR_M + r;
          S->gthr[r] = (rowthr && gi < nfit) ? __ldcg(rowthr + gi) : INF;
        }
      const bool ready = mbar_wait(&S->tfull[b], aph, abortf);
      tc_fence_after();
      __syncwarp();
      if (!bar_and(1, TC_EPI_WARPS * 32, ready)) { ok = false; break; }
      if (ntile++ == 0 && ew == 0 && lane == 0) {
        __threadfence_block();
        *(volatile int*)&S->thr_item = cur;  // this item's thresholds are live
      }
      const uint32_t tq = tbase + ((uint32_t)(q * 32) << 16) + b * 256;
      uint64_t* rowbuf = dense ? nullptr : candbuf + ((int64_t)grow * nseg + seg) * TC_CAPG;
#pragma unroll 1
      for (int ci = ci0; ci < ci1; ++ci) {
        float vx[8], vy[8], vz[8];
        tmem_ld8(tq + 8 * ci, vx);
        tmem_ld8(tq + TC_FR_N + 8 * ci, vy);
        tmem_ld8(tq + 2 * TC_FR_N + 8 * ci, vz);
        tmem_wait_ld();
#pragma unroll
        for (int g0 = 0; g0 < 8; g0 += 3) {
          // v[g][d]: row (f, c) of the Gram of pair (f, column frame g0+g)
          float v[3][3];
#pragma unroll
          for (int g = 0; g < 3; ++g) {
            v[g][0] = (g0 + g < 8) ? vx[(g0 + g) & 7] : 0.f;
            v[g][1] = (g0 + g < 8) ? vy[(g0 + g) & 7] : 0.f;
            v[g][2] = (g0 + g < 8) ? vz[(g0 + g) & 7] : 0.f;
          }
          // 3-lane transpose: lane (f, m=c) gathers rows 0..2 of block m
          float R[3][3];
#pragma unroll
          for (int d = 0; d < 3; ++d) R[0][d] = sel3(c, v[0][d], v[1][d], v[2][d]);
#pragma unroll
          for (int s = 1; s < 3; ++s) {
            const int src = 3 * f + (c + s) % 3;
            const int gi = (c + 3 - s) % 3;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              float send = sel3(gi, v[0][d], v[1][d], v[2][d]);
              R[s][d] = __shfl_sync(0xffffffffu, send, src & 31);
            }
          }
          // row (c + s) % 3 of block m is R[s]
          float G[9];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            G[0 + d] = sel3(c, R[0][d], R[2][d], R[1][d]) * ginv;
            G[3 + d] = sel3(c, R[1][d], R[0][d], R[2][d]) * ginv;
            G[6 + d] = sel3(c, R[2][d], R[1][d], R[0][d]) * ginv;
          }
          const int gl = 8 * ci + g0 + c;
          const int j = tile * TC_FR_N + gl;
          if (rowok && (g0 + c < 8) && j < Nr) {
            const float* cr = S->colrec + gl * MDS_REC;
            if (dense) {
              // (pivot bounds: no refinement, a loose bound only weakens a skip)
              const float sv = screen_shifted_f32(G, rrec, cr, nofit != 0, guard * (rrec[15] + cr[15]),
                                                  __builtin_huge_valf(), false);
              dense[(int64_t)j * nfit + grow] = sqrtf(fmaxf(sv, 0.0f));
            } else {
              const float thr = fminf(*(volatile float*)&S->thr[rloc], S->gthr[rloc]);
              float sv = screen_shifted_f32(G, rrec, cr, nofit != 0, guard * (rrec[15] + cr[15]), thr);
              sv = fmaxf(sv, 0.0f);
              if (sv < thr) {
                int pos = atomicAdd(&S->cnt[rloc], 1);
                if (pos < TC_CAPG)
                  rowbuf[pos] = mds_pack_key(sv, j);
                else
                  atomicMax(err, 4);  // cannot happen with K' + 160 <= capacity
              }
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S->tempty[b]);
      ++acc;
      if (dense) continue;
      bar_named(1, TC_EPI_WARPS * 32);  // every append of this tile is done
      // compaction of this warp's rows
      for (int fr = h; fr < 10; fr += 4) {
        const int r = q * 10 + fr;
        const int gr = rt * TC_FR_M + r;
        if (gr >= nfit) continue;
        // Cut back to K' as soon as TC_SLACK keys beyond K' have arrived: the
        // threshold then follows the K'-th bound closely, which is what the
        // skip test and the append filter run on.
        // With the (k+1)-th rule, a row without a threshold gets one as soon
        // as k+1 keys are there (no keys dropped while fewer than K').
        int n = S->cnt[r];
        const bool inf = S->thr[r] == INF;
        const bool need = n > Kp + TC_SLACK || (n > Kp && inf);
        const bool early = !need && nmax && inf && n >= k1;
        if (!need && !early) continue;
        uint64_t* src = candbuf + ((int64_t)gr * nseg + seg) * TC_CAPG;
        n = min(n, TC_CAPG);
        float tk1 = INF;
        float t = warp_select_keep2(src, n, TC_CAPG, 0, need ? Kp : 0, reinterpret_cast<int*>(scratch), lane,
                                    nmax ? k1 : 0, &tk1);
        if (nmax) t = fminf(t, tk1 + 2.0f * guard * (S->rowrec[r * MDS_REC + 15] + __ldg(nmax)));
        if (lane == 0) {
          if (need) S->cnt[r] = Kp;
          S->thr[r] = t;
          if (rowthr) atomicMin(reinterpret_cast<int*>(rowthr + gr), __float_as_int(t));  // t >= 0
        }
        __syncwarp();
      }
    }
    if (!ok && lane == 0) {
      atomicMax(err, 3);
      *abortf = 1;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tbase, TC_TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled_t)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                      const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                      CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                      CUtensorMapFloatOOBfill);

int encode_map(mds_ctx* ctx, CUtensorMap* map, const void* ptr, int rows, int Ap, int boxrows, unsigned prec) {
  static PFN_encodeTiled_t fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return mds_fail(ctx, MDS_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    fn = reinterpret_cast<PFN_encodeTiled_t>(p);
  }
  cuuint64_t gdim[2] = {(cuuint64_t)(2 * Ap), (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)(2 * Ap) * 2};
  cuuint32_t box[2] = {TC_KB, (cuuint32_t)boxrows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, prec == MDS_PREC_FP16X3 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                  2, const_cast<void*>(ptr), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return mds_fail(ctx, MDS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return MDS_OK;
}

int tc_choose_nseg(mds_ctx* ctx, const KnnRmsPlan& pl, int nfit) {
  int nrt = (nfit + TC_FR_M - 1) / TC_FR_M;
  int nct = (pl.nref + TC_FR_N - 1) / TC_FR_N;
  int best = 1;
  double besteff = 0;
  for (int s = 1; s <= 8 && s <= nct; ++s) {
    double w = (double)nrt * s / ctx->num_sms;
    double eff = w / std::ceil(w);
    if (eff > besteff + 0.02) {
      besteff = eff;
      best = s;
    }
    if (eff >= 0.97) break;
  }
  return best;
}

int tc_seg_stride() { return TC_CAPG; }

int launch_screen_tc(mds_ctx* ctx, const KnnRmsPlan& pl, const TcOperands& fit, const TcOperands& ref,
                     const float* recf, const float* recr, int nfit, int Kp, int nseg, uint64_t* cand,
                     int* cand_n, int* derr, const TcSkip* skip, float* dense, float* rowthr, const float* nmax,
                     unsigned long long* ntiles, int rt0, int nrt_items) {
  if (Kp + 2 * TC_FR_N > TC_CAPG)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "tensor-core screen supports K' <= %d (k too large)",
                    TC_CAPG - 2 * TC_FR_N);
  if (pl.Ap % TC_KB) return mds_fail(ctx, MDS_ERR_INTERNAL, "padded atom count not a multiple of %d", TC_KB);
  CUtensorMap mA, mB;
  MDS_TRY(encode_map(ctx, &mA, fit.A.p, fit.rowsA, pl.Ap, TC_M, pl.prec));
  MDS_TRY(encode_map(ctx, &mB, ref.B.p, ref.rowsB, pl.Ap, TC_N, pl.prec));
  // row tiles [rt0, rt0 + nrt) (dense mode may take a range; else all)
  const int nrt = (nrt_items >= 0) ? nrt_items : (nfit + TC_FR_M - 1) / TC_FR_M;
  if (rt0 && (&fit == &ref || !dense)) return mds_fail(ctx, MDS_ERR_INTERNAL, "row-tile range outside the pivot pass");
  const int nitems = nrt * nseg;
  if (nitems <= 0) return MDS_OK;
  const int grid = std::min(nitems, ctx->num_sms);
  const size_t smem = TC_SMEM_BYTES;
  static bool attr_set = false;  // set once: the call is also made while a stream is being captured
  if (!attr_set) {
    MDS_CUDA(ctx, cudaFuncSetAttribute(k_screen_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  // With an external error flag the caller checks it after the stream is
  // synchronised (the launch can then be captured in a CUDA graph).
  DevBuf err(ctx);
  int* e = derr;
  if (!e) {
    MDS_TRY(err.alloc(ctx, 2 * sizeof(int)));
    e = err.as<int>();
  }
  MDS_CUDA(ctx, cudaMemsetAsync(e, 0, 2 * sizeof(int), ctx->stream));  // error code, work counter
  if (rowthr)  // 0x7f7f7f7f = 3.4e38: above every bound
    MDS_CUDA(ctx, cudaMemsetAsync(rowthr, 0x7f, sizeof(float) * (size_t)nfit, ctx->stream));
  const float s = tc_scale(pl.prec);
  const uint32_t idesc = umma_idesc_f16(TC_M, TC_N, pl.prec == MDS_PREC_FP16X3 ? 0 : 1);
  const int stall = (ctx->inject & MDS_INJECT_SCREEN_STALL) ? 1 : 0;
  ctx->inject &= ~MDS_INJECT_SCREEN_STALL;
  ctx->stats.launches++;
  k_screen_tc<<<grid, TC_THREADS, smem, ctx->stream>>>(mA, mB, recf, recr, nfit, pl.nref, pl.Ap, pl.nofit,
                                                       pl.guard_tc, 1.0f / (s * s), idesc, Kp, nseg, nitems, rt0,
                                                       &fit == &ref ? 1 : 0, skip ? skip->pivlb : nullptr,
                                                       skip ? skip->prad : nullptr, skip ? skip->rowlo : nullptr,
                                                       skip ? skip->piv2 : 0, skip ? skip->far_perm : nullptr,
                                                       dense, rowthr, nmax, pl.k + 1, ntiles, cand, cand_n, e,
                                                       stall);
  MDS_CUDA(ctx, cudaGetLastError());
  if (derr) return MDS_OK;
  int herr = 0;
  MDS_CUDA(ctx, cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MDS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr) return mds_fail(ctx, MDS_ERR_TIMEOUT, "tensor-core screen: a bounded wait timed out (role %d)", herr);
  return MDS_OK;
}

// ---------------------------------------------------------------------------
// tile skipping: pivots, radii and the dense pivot pass
// ---------------------------------------------------------------------------
// copy the deviations and records of the frames idx[] (pivots)
__global__ void k_gather_frames(const float* __restrict__ A, const float* __restrict__ R, const int* __restrict__ idx,
                                int n, int Ap, float* __restrict__ Ao, float* __restrict__ Ro) {
  const int t = blockIdx.x;
  if (t >= n) return;
  const int f = idx[t];
  for (int e = threadIdx.x; e < 3 * Ap; e += blockDim.x) Ao[(int64_t)t * 3 * Ap + e] = A[(int64_t)f * 3 * Ap + e];
  for (int e = threadIdx.x; e < MDS_REC; e += blockDim.x) Ro[(int64_t)t * MDS_REC + e] = R[(int64_t)f * MDS_REC + e];
}

// prad[T] >= max over frames j of column tile T of RMSD(j, pivot T): the
// distance of the two superposed copies, |a_j - a_p| (one feasible
// superposition, so an upper bound of the minimum), rounded up.
__global__ void k_tile_radius(const float* __restrict__ A, int Nr, int Ap, const int* __restrict__ idx,
                              float* __restrict__ prad) {
  __shared__ float wmax[8];
  const int T = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float4* ap = reinterpret_cast<const float4*>(A + (int64_t)idx[T] * 3 * Ap);
  float best = 0.0f;
  for (int g = warp; g < TC_FR_N; g += blockDim.x >> 5) {
    const int j = T * TC_FR_N + g;
    if (j >= Nr) break;
    const float4* aj = reinterpret_cast<const float4*>(A + (int64_t)j * 3 * Ap);
    float acc = 0.0f;
    for (int q = lane; q < 3 * Ap / 4; q += 32) {
      const float4 u = __ldg(aj + q), v = __ldg(ap + q);
      const float d0 = u.x - v.x, d1 = u.y - v.y, d2 = u.z - v.z, d3 = u.w - v.w;
      acc = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, fmaf(d3, d3, acc))));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    best = fmaxf(best, acc);
  }
  if (lane == 0) wmax[warp] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, wmax[w]);
    prad[T] = sqrtf(m) * (1.0f + 1e-5f) + 1e-7f;  // FP32 sums: round up
  }
}

// Radii of a set screened against itself with row-tile pivots, one warp per
// frame j of [F0, F1): j lies in row tile R = j / TC_FR_M and column tile
// T = R / 2, with the pivots p_2T and p_2T+1 (idx). rrad[R] bounds
// RMSD(i, p_R) over the row tile; prad[2T] and prad[2T+1] bound the
// distances of the column tile's frames to p_2T and p_2T+1. All zeroed
// beforehand and raised by atomicMax (non-negative floats order as their
// bits); the rounding up as above is monotonic, so the maximum of the
// rounded values is the rounded maximum.
__global__ void k_tile_radius_rc(const float* __restrict__ A, int N, int Ap, const int* __restrict__ idx, int nR,
                                 int F0, int F1, float* __restrict__ prad, float* __restrict__ rrad) {
  static_assert(TC_FR_N == 2 * TC_FR_M, "a column tile is two row tiles");
  const int lane = threadIdx.x & 31;
  const int j = F0 + (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (j >= F1 || j >= N) return;
  const int R = j / TC_FR_M, T = R / 2;
  const bool hasb = 2 * T + 1 < nR;
  const float4* pa = reinterpret_cast<const float4*>(A + (int64_t)idx[2 * T] * 3 * Ap);
  const float4* pb = reinterpret_cast<const float4*>(A + (int64_t)idx[hasb ? 2 * T + 1 : 2 * T] * 3 * Ap);
  const float4* aj = reinterpret_cast<const float4*>(A + (int64_t)j * 3 * Ap);
  float ac = 0.0f, ar = 0.0f;
  for (int q = lane; q < 3 * Ap / 4; q += 32) {
    const float4 u = __ldg(aj + q), v = __ldg(pa + q), w = __ldg(pb + q);
    float d0 = u.x - v.x, d1 = u.y - v.y, d2 = u.z - v.z, d3 = u.w - v.w;
    ac = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, fmaf(d3, d3, ac))));
    d0 = u.x - w.x, d1 = u.y - w.y, d2 = u.z - w.z, d3 = u.w - w.w;
    ar = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, fmaf(d3, d3, ar))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    ac += __shfl_xor_sync(0xffffffffu, ac, o);
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
  }
  if (lane == 0) {
    const float ra = sqrtf(ac) * (1.0f + 1e-5f) + 1e-7f, rb = sqrtf(ar) * (1.0f + 1e-5f) + 1e-7f;
    atomicMax(reinterpret_cast<int*>(rrad + R), __float_as_int(R == 2 * T ? ra : rb));
    atomicMax(reinterpret_cast<int*>(prad + 2 * T), __float_as_int(ra));
    if (hasb) atomicMax(reinterpret_cast<int*>(prad + 2 * T + 1), __float_as_int(rb));
  }
}

// rowlo[R][T] = min over the frames j of column tile T of lb(j, row pivot R)
// (row R of the dense pass) minus the row tile's radius: one warp per (R, T).
__global__ void k_row_lo(const float* __restrict__ lb, int N, int nC, int nR, const float* __restrict__ rrad,
                         float* __restrict__ rowlo) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nR * nC) return;
  const int R = w / nC, T = w % nC;
  const float* row = lb + (int64_t)R * N;
  float m = INFINITY;
  for (int j = T * TC_FR_N + lane; j < min(N, (T + 1) * TC_FR_N); j += 32) m = fminf(m, __ldg(row + j));
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) rowlo[w] = m - __ldg(rrad + R);
}

// *out = max over frames of rec[15] = |a|^2 (out zeroed beforehand;
// non-negative floats order as their bits).
__global__ void k_rec_nmax(const float* __restrict__ rec, int n, float* __restrict__ out) {
  float m = 0.0f;
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x)
    m = fmaxf(m, __ldg(rec + (int64_t)f * MDS_REC + 15));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(out), __float_as_int(m));
}

int tc_rec_nmax(mds_ctx* ctx, const float* rec, int n, float* out) {
  MDS_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(float), ctx->stream));
  ctx->stats.launches++;
  k_rec_nmax<<<std::max(1, std::min((n + 255) / 256, 2 * ctx->num_sms)), 256, 0, ctx->stream>>>(rec, n, out);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

// Pivots of a reference set, their operands and records, and the radii:
// once per reference set. By default the middle frame of every column tile
// (nP = nC pivots, prad[T] the tile's radius). With rowpiv (a set screened
// against itself) the middle frame of every row tile of TC_FR_M frames
// instead (nP = row tiles): prad[2T], prad[2T+1] bound column tile T's
// distances to its two row pivots and rrad[R] row tile R's radius.
int tc_pivots_begin(mds_ctx* ctx, const KnnRmsPlan& pl, TcPivots& pv, bool rowpiv) {
  const int Nr = pl.nref, Ap = pl.Ap;
  const int nC = (Nr + TC_FR_N - 1) / TC_FR_N;
  const int nR = (Nr + TC_FR_M - 1) / TC_FR_M;
  const int nP = rowpiv ? nR : nC;
  cudaStream_t s = ctx->stream;
  pv.hidx.resize(nP);
  if (rowpiv)
    for (int R = 0; R < nR; ++R) pv.hidx[R] = R * TC_FR_M + std::min(TC_FR_M, Nr - R * TC_FR_M) / 2;
  else
    for (int T = 0; T < nC; ++T) pv.hidx[T] = std::min(T * TC_FR_N + TC_FR_N / 2, Nr - 1);
  MDS_TRY(pv.idx.alloc(ctx, sizeof(int) * nP));
  MDS_TRY(pv.A.alloc(ctx, sizeof(float) * 3 * Ap * (size_t)nP));
  MDS_TRY(pv.R.alloc(ctx, sizeof(float) * MDS_REC * (size_t)nP));
  MDS_TRY(pv.rad.alloc(ctx, sizeof(float) * (rowpiv ? 2 * nC : nC)));
  if (rowpiv) MDS_TRY(pv.rrad.alloc(ctx, sizeof(float) * nR));
  // (pv.hidx lives until pv is destroyed, after the stream has used it)
  MDS_CUDA(ctx, cudaMemcpyAsync(pv.idx.p, pv.hidx.data(), sizeof(int) * nP, cudaMemcpyHostToDevice, s));
  if (rowpiv) {
    MDS_CUDA(ctx, cudaMemsetAsync(pv.rad.p, 0, sizeof(float) * 2 * nC, s));
    MDS_CUDA(ctx, cudaMemsetAsync(pv.rrad.p, 0, sizeof(float) * nR, s));
  }
  pv.nC = nC;
  pv.nP = nP;
  pv.rowpiv = rowpiv;
  return MDS_OK;
}

int tc_pivots_operand(mds_ctx* ctx, const KnnRmsPlan& pl, TcPivots& pv) {
  KnnRmsPlan pp = pl;
  pp.nref = pv.nP;
  return tc_prepare(ctx, pp, pv.A.as<float>(), pv.nP, pv.tc, 1);
}

int tc_pivots_radii(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Ar, TcPivots& pv, int f0, int f1) {
  if (!pv.rowpiv) return mds_fail(ctx, MDS_ERR_INTERNAL, "radii by row-tile range need row-tile pivots");
  // row tiles [R0, R1) hold frames [f0, f1); f0 starts a column tile, so the
  // frames of each column tile T and its pivots 2T, 2T+1 are all in range
  if (f0 % TC_FR_N) return mds_fail(ctx, MDS_ERR_INTERNAL, "radii range starts inside a column tile");
  f1 = std::min(f1, pl.nref);
  if (f1 <= f0) return MDS_OK;
  ctx->stats.launches++;
  k_tile_radius_rc<<<(f1 - f0 + 7) / 8, 256, 0, ctx->stream>>>(Ar, pl.nref, pl.Ap, pv.idx.as<int>(), pv.nP, f0, f1,
                                                               pv.rad.as<float>(), pv.rrad.as<float>());
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

int tc_skip_pivots(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Ar, const float* Rr, TcPivots& pv, bool rowpiv) {
  MDS_TRY(tc_pivots_begin(ctx, pl, pv, rowpiv));
  cudaStream_t s = ctx->stream;
  ctx->stats.launches++;
  k_gather_frames<<<pv.nP, 128, 0, s>>>(Ar, Rr, pv.idx.as<int>(), pv.nP, pl.Ap, pv.A.as<float>(), pv.R.as<float>());
  MDS_CUDA(ctx, cudaGetLastError());
  if (rowpiv) {
    MDS_TRY(tc_pivots_radii(ctx, pl, Ar, pv, 0, pl.nref));
  } else {
    ctx->stats.launches++;
    k_tile_radius<<<pv.nC, 256, 0, s>>>(Ar, pl.nref, pl.Ap, pv.idx.as<int>(), pv.rad.as<float>());
    MDS_CUDA(ctx, cudaGetLastError());
  }
  return tc_pivots_operand(ctx, pl, pv);
}

// Lower bounds of RMSD from every fit frame to every pivot (the screen in
// dense mode over the pivots) into lb [nP][nfit]; with f1 > 0 only for the
// fit frames [f0, f1) (f0 a multiple of the row tile). With derr (2 ints)
// the call does not synchronise and can be captured in a CUDA graph.
int tc_skip_bounds(mds_ctx* ctx, const KnnRmsPlan& pl, const TcOperands& fit, const float* recf, int nfit,
                   const TcPivots& pv, float* lb, int* derr, int f0, int f1) {
  KnnRmsPlan pp = pl;
  pp.nref = pv.nP;
  if (f1 <= 0) {
    f0 = 0;
    f1 = nfit;
  }
  if (f0 % TC_FR_M) return mds_fail(ctx, MDS_ERR_INTERNAL, "pivot pass range starts inside a row tile");
  const int rt0 = f0 / TC_FR_M;
  const int nrt = (std::min(f1, nfit) + TC_FR_M - 1) / TC_FR_M - rt0;
  if (nrt <= 0) return MDS_OK;
  // column segments (no lists in dense mode) so that there are >= 4 items per SM
  const int nct = (pv.nP + TC_FR_N - 1) / TC_FR_N;
  const int nseg = std::max(1, std::min(nct, (4 * ctx->num_sms + nrt - 1) / nrt));
  return launch_screen_tc(ctx, pp, fit, pv.tc, recf, pv.R.as<float>(), nfit, 32, nseg, nullptr, nullptr, derr,
                          nullptr, lb, nullptr, nullptr, nullptr, rt0, nrt);
}

// The row-tile bounds of a set screened against itself (pivots with rowpiv,
// lb [nR][n] from tc_skip_bounds): rowlo [nR][nC].
// Order of the non-diagonal items (row tile R, other segment s'), heaviest
// estimate first. Estimate: with t_R = twice the smallest bound from pivot R
// to another pivot (a scale of R's neighbour distances), the number of
// column tiles T of the segment with rowlo[R][T] < t_R. est[k] and a
// histogram first (one warp per row tile), then a descending exclusive scan
// of the histogram, then a scatter (order within one estimate unspecified:
// the results do not depend on the order of the items).
#define TC_EST_BUCKETS 1024
__global__ void k_far_est(const float* __restrict__ lb, const float* __restrict__ rowlo, int N, int nR, int nC,
                          int nseg, int* __restrict__ est, int* __restrict__ hist) {
  const int R = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (R >= nR) return;
  const int pf = R * TC_FR_M + min(TC_FR_M, N - R * TC_FR_M) / 2;  // pivot frame of R
  float m = INFINITY;
  for (int r2 = lane; r2 < nR; r2 += 32)
    if (r2 != R) m = fminf(m, __ldg(lb + (int64_t)r2 * N + pf));
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const float t = 2.0f * m;
  const int sd = diag_seg(R, nseg, nC);
  for (int sp = 0; sp < nseg - 1; ++sp) {
    const int seg = sp < sd ? sp : sp + 1;
    const int t0 = (int)((int64_t)nC * seg / nseg), t1 = (int)((int64_t)nC * (seg + 1) / nseg);
    int c = 0;
    for (int T = t0 + lane; T < t1; T += 32) c += (__ldg(rowlo + (int64_t)R * nC + T) < t) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    c = min(c, TC_EST_BUCKETS - 1);
    if (lane == 0) {
      est[R * (nseg - 1) + sp] = c;
      atomicAdd(hist + c, 1);
    }
  }
}

__global__ void k_far_scan(const int* __restrict__ hist, int* __restrict__ off) {
  // one block of TC_EST_BUCKETS threads: off[v] = number of items with est > v
  __shared__ int sh[TC_EST_BUCKETS];
  const int v = threadIdx.x;
  sh[v] = hist[TC_EST_BUCKETS - 1 - v];  // descending order of v
  __syncthreads();
  for (int o = 1; o < TC_EST_BUCKETS; o <<= 1) {
    const int add = (v >= o) ? sh[v - o] : 0;
    __syncthreads();
    sh[v] += add;
    __syncthreads();
  }
  const int inc = sh[v];                               // items with est >= TC_EST_BUCKETS-1-v
  off[TC_EST_BUCKETS - 1 - v] = inc - hist[TC_EST_BUCKETS - 1 - v];
}

__global__ void k_far_scatter(const int* __restrict__ est, int nfar, const int* __restrict__ off,
                              int* __restrict__ cnt, int* __restrict__ perm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nfar) return;
  const int e = est[k];
  perm[off[e] + atomicAdd(cnt + e, 1)] = k;
}

int tc_far_order(mds_ctx* ctx, const TcPivots& pv, const float* lb, const float* rowlo, int n, int nseg,
                 int* work, int* perm) {
  // work: 3 * TC_EST_BUCKETS + nR * (nseg - 1) ints
  if (!pv.rowpiv || nseg < 2) return mds_fail(ctx, MDS_ERR_INTERNAL, "far order needs row pivots and segments");
  const int nR = pv.nP, nfar = nR * (nseg - 1);
  int* hist = work;
  int* off = work + TC_EST_BUCKETS;
  int* cnt = work + 2 * TC_EST_BUCKETS;
  int* est = work + 3 * TC_EST_BUCKETS;
  cudaStream_t s = ctx->stream;
  MDS_CUDA(ctx, cudaMemsetAsync(work, 0, sizeof(int) * 3 * TC_EST_BUCKETS, s));
  ctx->stats.launches += 3;
  k_far_est<<<(nR + 7) / 8, 256, 0, s>>>(lb, rowlo, n, nR, pv.nC, nseg, est, hist);
  k_far_scan<<<1, TC_EST_BUCKETS, 0, s>>>(hist, off);
  k_far_scatter<<<(nfar + 255) / 256, 256, 0, s>>>(est, nfar, off, cnt, perm);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

int tc_skip_rowlo(mds_ctx* ctx, const TcPivots& pv, const float* lb, int n, float* rowlo) {
  if (!pv.rowpiv) return mds_fail(ctx, MDS_ERR_INTERNAL, "row-tile pivots were not built");
  const int nR = pv.nP;
  const int warps = nR * pv.nC;
  ctx->stats.launches++;
  k_row_lo<<<(warps + 7) / 8, 256, 0, ctx->stream>>>(lb, n, pv.nC, nR, pv.rrad.as<float>(), rowlo);
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}
