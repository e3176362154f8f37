// knn_data_tc.cu -- the all-pairs candidate screen of knn_data on the 5th
// generation tensor cores (precision flag MDS_PREC_BF16X3).
//
// x.y is one GEMM of the vectors split into BF16 parts, x = hi + lo:
// hi.hi + hi.lo + lo.hi, FP32 accumulation in TMEM. The screen value of a
// pair is a lower bound of its squared distance,
//   Euclidean:   |x|^2 + |y|^2 - 2 x.y - c (|x|^2 + |y|^2)
//   correlation: (1 - z_x.z_y) / 2     - c (|z_x|^2 + |z_y|^2)
// (z: standardised vectors, |z| = 1; c = MDS_GUARD_TC covers the rounding of
// the split products and of the FP32 operands).
//
// Work item = (row pair tile of 256 fit vectors, column segment). The row
// pair tile stays resident in shared memory for the whole item (two 128-row
// MMA operands); reference vectors stream through a 3-4 stage TMA pipeline in
// tiles of 128 (64-byte swizzle, K-blocks of 32 dimensions). Per tile the MMA
// warp writes two 128 x 128 FP32 accumulators; TMEM holds two such pairs
// (512 columns) so the epilogue of one tile overlaps the MMAs of the next.
// Warp 0 claims items from a global counter, loads the resident rows and the
// reference tiles and publishes (item, tile) tasks in a ring; warp 1 issues
// the MMAs; 16 epilogue warps, a pair per 32 rows (one warp per column
// half), append the pairs below the row's threshold to the row's list in
// global memory: each (row, column half) owns a region of the list and
// counts in a register, so an append is a compare and a store. When a
// region nears full, the warp owning the row cuts its two regions back to
// K' by a warp radix select. Rows share their thresholds across column
// segments through rowthr. Every mbarrier wait is bounded; the two warps of
// a pair synchronise on their own hardware named barrier, which carries each
// wait's outcome, so on a timeout all roles leave together: the kernel
// records an error, drains, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "knn_common.cuh"
#include "tc_ptx.cuh"
#include "tc_select.cuh"

#define TV_ROWS 256         // fit vectors per work item (two MMA row tiles)
#define TV_N 128            // reference vectors per column tile
#define TV_KB 32            // dimensions per K-block (64-byte rows)
#define TV_THREADS 576      // producer, MMA, 16 epilogue warps
#define TV_EPI 16
#define TV_SUB_BYTES 8192   // one 128-row x 32-dimension BF16 operand tile
#define TV_STAGE_BYTES (2 * TV_SUB_BYTES)  // reference hi + lo of one K-block
#define TV_MAXST 4
#define TV_TQ 8
#define TV_SCR 512          // words of per-warp shared scratch: 16 columns x 32 lanes of screen values, or
                            // the radix histogram of a compaction (256 ints)
#define TV_LCAP 256         // keys per (row, column half) list region; a row's list is 2 regions
#define TV_MAX_DP 128
#define TV_PILOT 16         // column tiles each row pair visits in the threshold-seeding pass
#define TV_KHMAX 96         // largest k + 1 with threshold heaps in the epilogue

// FP32 vectors [n][Dp] -> BF16 split rows [rows][hi(Dp) | lo(Dp)], rows
// beyond n zero. With terms != nullptr also the column term of each row as a
// reference vector (the screen value is row term + column term - 2 x.y, or
// - x.y/2 for correlation): |y|^2 (1 - c), or -c |y|^2; +inf beyond n.
// With nmax != nullptr (zeroed by the caller) also the largest norm of the n
// vectors, as the float's bits (norms are non-negative). perm (or null): row
// r is vector perm[r] (the locality order of vec_order.cu); nsorted (or
// null) receives the norms in that order. devn (or null; correlation): the
// largest | |z|^2 - 1 | of the standardised vectors, as the float's bits.
__global__ void k_vec_split(const float* __restrict__ X, int n, int Dp, int rows, __nv_bfloat16* __restrict__ out,
                            const float* __restrict__ nrm, float guard, int corr, float* __restrict__ terms,
                            float* __restrict__ nmax, const int* __restrict__ perm, float* __restrict__ nsorted,
                            unsigned* __restrict__ devn) {
  const int64_t total = (int64_t)rows * Dp;
  float mx = 0.0f, dv = 0.0f;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / Dp;
    const int d = (int)(e % Dp);
    const int64_t src = (r < n && perm) ? (int64_t)perm[r] : r;
    if (nmax && d == 0 && r < n) mx = fmaxf(mx, nrm[src]);
    if (nsorted && d == 0 && r < n) nsorted[r] = nrm[src];
    if (devn && d == 0 && r < n) dv = fmaxf(dv, fabsf(nrm[src] - 1.0f));
    if (terms && d == 0)
      terms[r] = (r < n) ? (corr ? -guard * nrm[src] : nrm[src] * (1.0f - guard)) : __int_as_float(0x7f800000);
    const float x = (r < n) ? X[src * Dp + d] : 0.0f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(x);
    const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
    out[r * 2 * Dp + d] = hi;
    out[r * 2 * Dp + Dp + d] = lo;
  }
  if (nmax) {
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(reinterpret_cast<int*>(nmax), __float_as_int(mx));
  }
  if (devn) {
    for (int o = 16; o > 0; o >>= 1) dv = fmaxf(dv, __shfl_xor_sync(0xffffffffu, dv, o));
    if ((threadIdx.x & 31) == 0 && dv > 0.0f) atomicMax(devn, __float_as_uint(dv));
  }
}

struct TvShared {
  uint64_t full[TV_MAXST], empty[TV_MAXST], tfull[2], tempty[2], afull, aempty, done;
  uint64_t tq_full[TV_TQ], tq_empty[TV_TQ];
  int2 task[TV_TQ];
  uint32_t tmem_base;
  int abortf;
  int cnt2[TV_ROWS][2];   // keys in each (row, column half) region
  float thr[TV_ROWS];     // the row's list threshold (+inf until its list first holds k+1 keys)
  float rslack[TV_ROWS][2];  // 2 g (|x|^2 + nmax): the (k+1)-th bound's slack of the row
};

static size_t tv_smem_bytes(int Dp, int nst, int KH) {
  return (size_t)TV_ROWS * 2 * Dp * 2 + (size_t)nst * TV_STAGE_BYTES + sizeof(TvShared) +
         (size_t)TV_EPI * TV_SCR * 4 + (size_t)TV_ROWS * 2 * KH * 2 + 1024;
}

// The (row, column half) heaps of the epilogue: the KH smallest bounds the
// half has appended, as the upper 16 bits of the non-negative float rounded
// up (so a heap value is never below the bound it stands for), in a max-heap
// whose root is the half's KH-th smallest; 0x7F80 (+inf) marks a free slot.
__device__ __forceinline__ uint16_t tv_u16_up(float b) {
  const uint32_t u = __float_as_uint(b);
  return (uint16_t)((u >> 16) + ((u & 0xFFFFu) ? 1u : 0u));
}
__device__ __forceinline__ float tv_u16_float(uint32_t h) { return __uint_as_float(h << 16); }
// Replaces the root by v when v is smaller, restoring the heap; the root is
// written once, with the new maximum, so a concurrent reader of the root sees
// either the old or the new k1-th value.
__device__ __forceinline__ void tv_heap_push(uint16_t* hp, int n, uint16_t v) {
  if (v >= hp[0]) return;
  int i = 0;
  while (true) {
    const int l = 2 * i + 1;
    if (l >= n) break;
    int c = l;
    uint16_t cv = hp[l];
    if (l + 1 < n) {
      const uint16_t rv = hp[l + 1];
      if (rv > cv) {
        c = l + 1;
        cv = rv;
      }
    }
    if (cv <= v) break;
    hp[i] = cv;
    i = c;
  }
  hp[i] = v;
}

// Column tiles of a segment [t0, t1) in visiting order: outward from td.
__device__ __forceinline__ int tv_tile_order(int i, int t0, int t1, int td) {
  const int L = td - t0, Rn = t1 - 1 - td, m = min(L, Rn);
  if (i == 0) return td;
  if (i <= 2 * m) return (i & 1) ? td + (i + 1) / 2 : td - i / 2;
  const int j = i - 2 * m;
  return (Rn > L) ? td + m + j : td - m - j;
}


// Work item -> (row pair tile, segment). In locality order (near_first) the
// segment holding each row pair tile's start tile comes first: items [0, nrp)
// are those segments, items [nrp, nrp * nseg) the others. By the time a row
// pair's far segments are claimed its near segment has set the rows'
// thresholds, and most far tiles are skipped. Start tile: the diagonal's
// (diag) or tdall[rp].
__device__ __forceinline__ int2 tv_item(int item, int nseg, int nrp, int ncoltiles, int near_first, int diag,
                                        const int* tdall) {
  if (!near_first || nseg == 1) return make_int2(item / nseg, item % nseg);
  const int rp = item < nrp ? item : (item - nrp) / (nseg - 1);
  const int tstart = diag ? min((rp * TV_ROWS + TV_ROWS / 2) / TV_N, ncoltiles - 1) : __ldg(tdall + rp);
  int near = 0;
  while (near + 1 < nseg && (int)((int64_t)ncoltiles * (near + 1) / nseg) <= tstart) ++near;
  if (item < nrp) return make_int2(rp, near);
  const int j = (item - nrp) % (nseg - 1);
  return make_int2(rp, j < near ? j : j + 1);
}

// One fit row's list (regions src[0, c0) and src[lcap, lcap + c1)): keep
// the Kp best, drop those above the row's threshold tp (appended under a
// looser one: every pair the screen left out lies at or above the final
// threshold, which the recheck verifies against), and write the rest,
// unsorted, as the segment's candidate list (the recheck sorts the merged
// lists), with the column indices mapped through cperm when the columns are
// in locality order. Called by the warp owning the row.
__device__ __forceinline__ void tv_publish(uint64_t* src, int c0, int c1, int lcap, int Kp, float tp, int* hist,
                                           uint64_t* dst, int* dst_n, int lane, const int* cperm) {
  if (c0 + c1 > Kp) {
    warp_select_keep2(src, c0, lcap, c1, Kp, hist, lane);
    c0 = Kp;
    c1 = 0;
  }
  int m = 0;
  for (int r = 0; r < 2; ++r) {
    const int n = r ? c1 : c0;
    const uint64_t* from = src + (r ? lcap : 0);
    for (int x0 = 0; x0 < n; x0 += 32) {
      const int x = x0 + lane;
      const uint64_t key = (x < n) ? from[x] : MDS_KEY_INF;
      const bool keep = x < n && mds_key_value(key) <= tp;
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep)
        dst[m + __popc(bal & ((1u << lane) - 1u))] =
            cperm ? mds_pack_key(mds_key_value(key), __ldg(cperm + mds_key_index(key))) : key;
      m += __popc(bal);
    }
  }
  if (lane == 0) *dst_n = m;
  __syncwarp();
}

__global__ void __launch_bounds__(TV_THREADS, 1)
k_screen_tcv(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
             const float* __restrict__ nf, const float* __restrict__ colterm, int nfit, int Nr, int Dp, int nst,
             int corr, float guard, uint32_t idesc, int Kp, int nseg, int nitems, int diag, int pilot,
             float* __restrict__ rowthr, uint64_t* __restrict__ work, uint64_t* __restrict__ candout,
             int* __restrict__ cand_n, int* __restrict__ err, int lcap, int k1, const float* __restrict__ nmax,
             const float* __restrict__ dlo, const int* __restrict__ tdv, const int* __restrict__ tdall,
             int near_first, const int* __restrict__ rperm, const int* __restrict__ cperm, int KH,
             const unsigned* __restrict__ devn) {
  // err[0]: error code; err[1]: next unclaimed work item (zeroed by the host);
  // err[2]: column tiles computed (added to).
  // Locality order (vec_order.cu; all four null without it): rows and columns
  // are in sorted order, rperm/cperm map them to the original indices, which
  // the published lists carry (rowthr stays in sorted order). dlo [row pair
  // tile][column tile]: the lower bound of the distance of the tile's pairs;
  // the producer skips a tile when dlo^2 is at least the largest threshold of
  // the item's rows. tdv: the visit's start tile ([item] for the pilot,
  // [row pair tile][segment] otherwise) when the set is not screened against
  // itself, tdall [row pair tile] the start over all tiles; near_first: the
  // item order of tv_item. For the correlation metric (devn != null) dlo
  // bounds |z_x - z_y| of the standardised vectors, and the distance is
  // |z_x - z_y|^2 / 4 within corr_margin.
  // KH = ceil(k1 / 2) (or 0: off): the epilogue keeps, per (row, column half),
  // a heap of the KH smallest bounds it appended (tv_heap_push), so the row's
  // threshold follows the larger of its halves' KH-th bounds (2 KH >= k1
  // bounds lie at or below it) plus the slack, with no search of the list;
  // the list is searched only to cut it back. (Heaps of k1 per half with the
  // smaller root: one level deeper, and a half's k1-th is looser.)
  // pilot > 0: a pass that only seeds rowthr: each item (one per row pair
  // tile, nseg = 1) visits `pilot` column tiles (outward from the diagonal
  // for a set against itself, else spread over the set) and lowers each
  // row's rowthr to the K'-th smallest screen value it saw, an upper bound of
  // the row's final K'-th smallest; nothing else is written.
  // colterm: [ncoltiles * TV_N] column terms (+inf past Nr).
  // work: [gridDim.x][TV_ROWS][TC_CAPG] list buffers of the CTAs; a row's
  // list is two regions of lcap keys (K' + one tile's half, rounded up): a
  // smaller region keeps the CTAs' lists resident in L2.
  // candout: [nfit][nseg][Kp] lists, cand_n [nfit][nseg] their sizes.
  // Thresholds from the (k+1)-th bound (nmax: the largest norm term of the
  // reference set): a key's value b is the screen value minus the guard
  // g (|x|^2 + |y|^2), and the screen value is within the guard of the exact
  // one, so the row's (k+1)-th exact value is at most b_(k+1) +
  // 2 g (|x|^2 + nmax); a compaction sets the row threshold to the smaller of
  // that and the K'-th bound, and the first one runs when k1 keys arrive.
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  const int nkb = Dp / TV_KB;
  unsigned char* arows = base;                                   // [2][nkb][hi, lo] 8 KB tiles
  unsigned char* stages = base + (size_t)TV_ROWS * 2 * Dp * 2;   // nst x (hi, lo)
  TvShared* S = reinterpret_cast<TvShared*>(stages + (size_t)nst * TV_STAGE_BYTES);
  int* scratch_all = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(S) + sizeof(TvShared));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncoltiles = (Nr + TV_N - 1) / TV_N;
  const float INF = __int_as_float(0x7f800000);

  if (threadIdx.x == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&S->full[s], 1);
      mbar_init(&S->empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&S->tfull[b], 1);
      mbar_init(&S->tempty[b], TV_EPI);
    }
    mbar_init(&S->afull, 1);
    mbar_init(&S->aempty, 1);
    mbar_init(&S->done, 1);
    for (int i = 0; i < TV_TQ; ++i) {
      mbar_init(&S->tq_full[i], 1);
      mbar_init(&S->tq_empty[i], 1 + TV_EPI);
    }
    S->abortf = 0;
    mbar_fence_init();
  }
  for (int r = threadIdx.x; r < TV_ROWS; r += blockDim.x) {
    S->cnt2[r][0] = 0;
    S->cnt2[r][1] = 0;
    S->thr[r] = INF;
  }
  uint16_t* heaps = reinterpret_cast<uint16_t*>(scratch_all + TV_EPI * TV_SCR);  // [TV_ROWS][2][KH]
  for (int e = threadIdx.x; e < TV_ROWS * 2 * KH; e += blockDim.x) heaps[e] = 0x7F80;
  if (warp == 1) {
    tmem_alloc(&S->tmem_base, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = S->tmem_base;
  volatile int* abortf = &S->abortf;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // Lane 0 claims items, issues the copies and publishes the tasks; with
    // tile bounds the whole warp decides, 32 visit steps at a time, which
    // tiles to skip.
    uint32_t stage = 0, phase = 0, qs = 0, na = 0;
    int ok = 1, nvis = 0;
    if (lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
    }
    auto push = [&](int item, int tile) -> bool {
      const uint32_t slot = qs % TV_TQ, ph = (qs / TV_TQ) & 1;
      ++qs;
      if (!mbar_wait(&S->tq_empty[slot], ph ^ 1, abortf, 1000000000ull, 1024)) return false;
      S->task[slot] = make_int2(item, tile);
      mbar_arrive(&S->tq_full[slot]);
      return true;
    };
    while (ok) {
      int item = 0;
      if (lane == 0) item = atomicAdd(err + 1, 1);
      item = __shfl_sync(0xffffffffu, item, 0);
      if (item >= nitems) {
        if (lane == 0) ok = push(-1, -1);
        break;
      }
      const int2 rs = tv_item(item, nseg, nitems / nseg, ncoltiles, near_first, diag, tdall);
      const int rp = rs.x, seg = rs.y;
      const int t0 = pilot ? 0 : (int)((int64_t)ncoltiles * seg / nseg);
      const int t1 = pilot ? ncoltiles : (int)((int64_t)ncoltiles * (seg + 1) / nseg);
      const int nvisit = pilot ? pilot : t1 - t0;
      const int td = diag ? min(max((rp * TV_ROWS + TV_ROWS / 2) / TV_N, t0), t1 - 1)
                          : (tdv ? min(max(__ldg(tdv + (pilot ? rp : rp * nseg + seg)), t0), t1 - 1) : t0);
      const bool spread = pilot && !diag && !tdv;
      // the resident rows: wait until the MMAs of the previous item are done
      if (lane == 0) {
        if (na > 0 && !mbar_wait(&S->aempty, (na - 1) & 1, abortf, 1000000000ull, 1024)) {
          ok = 0;
        } else {
          mbar_expect_tx(&S->afull, (uint32_t)(TV_ROWS * 2 * Dp * 2));
          for (int u = 0; u < 2; ++u)
            for (int kb = 0; kb < nkb; ++kb)
              for (int p = 0; p < 2; ++p)
                tma_load_2d(arows + (size_t)((u * nkb + kb) * 2 + p) * TV_SUB_BYTES, &tmA, &S->afull,
                            p * Dp + kb * TV_KB, (2 * rp + u) * 128);
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      ++na;
      const float* dl = (dlo && !pilot) ? dlo + (int64_t)rp * ncoltiles : nullptr;
      const float dsc = devn ? 0.25f : 1.0f;
      const float dmarg = devn ? corr_margin(devn, Dp) : 0.0f;
      for (int base = 0; base < nvisit && ok; base += 32) {
        unsigned skip = 0u;
        if (dl) {
          // the largest threshold of the item's rows now (rowthr holds each
          // row's smallest, its own list's included)
          float mx = 0.0f;
          for (int x = lane; x < TV_ROWS; x += 32) {
            const int gx = rp * TV_ROWS + x;
            if (gx < nfit) mx = fmaxf(mx, __ldcg(rowthr + gx));
          }
          for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
          bool sk = false;
          if (base + lane < nvisit) {
            const float b = __ldg(dl + tv_tile_order(base + lane, t0, t1, td));
            sk = b > 0.0f && b * b * dsc - dmarg >= mx;
          }
          skip = __ballot_sync(0xffffffffu, sk);
        }
        if (lane == 0) {
          const int nb = min(32, nvisit - base);
          for (int i = 0; i < nb && ok; ++i) {
            if ((skip >> i) & 1u) continue;
            const int ti = base + i;
            const int tile = spread ? (int)((int64_t)ti * ncoltiles / pilot) : tv_tile_order(ti, t0, t1, td);
            if (!(ok = push(item, tile))) break;
            ++nvis;
            for (int kb = 0; kb < nkb; ++kb) {
              if (!mbar_wait(&S->empty[stage], phase ^ 1, abortf, 1000000000ull, 1024)) { ok = 0; break; }
              unsigned char* st = stages + stage * TV_STAGE_BYTES;
              mbar_expect_tx(&S->full[stage], TV_STAGE_BYTES);
              tma_load_2d(st, &tmB, &S->full[stage], kb * TV_KB, tile * TV_N);
              tma_load_2d(st + TV_SUB_BYTES, &tmB, &S->full[stage], Dp + kb * TV_KB, tile * TV_N);
              if (++stage == (uint32_t)nst) { stage = 0; phase ^= 1; }
            }
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
      }
      if (!ok) break;
      if (lane == 0) ok = push(item, -1);
      ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    if (lane == 0) {
      if (nvis) atomicAdd(err + 2, nvis);
      if (!ok) {
        atomicMax(err, 1);
        *abortf = 1;
        // let the copies in flight land before the CTA exits
        volatile int dummy = 0;
        if (na > 0) mbar_wait(&S->afull, (na - 1) & 1, &dummy, 50000000ull);
        for (int s = 0; s < nst; ++s) mbar_wait(&S->full[s], 0, &dummy, 50000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      uint32_t stage = 0, phase = 0, acc = 0, na = 0;
      int cur = -1;
      bool ok = true;
      const uint32_t abase = smem_u32(arows), sbase = smem_u32(stages);
      for (uint32_t qs = 0; ok; ++qs) {
        const uint32_t slot = qs % TV_TQ, qph = (qs / TV_TQ) & 1;
        if (!mbar_wait(&S->tq_full[slot], qph, abortf, 1000000000ull, 64)) { ok = false; break; }
        const volatile int* tv = reinterpret_cast<volatile int*>(&S->task[slot]);
        const int2 t = make_int2(tv[0], tv[1]);
        mbar_arrive(&S->tq_empty[slot]);
        if (t.x < 0) break;
        if (t.x != cur) {  // a new item's rows (consumed even when every tile was skipped)
          cur = t.x;
          if (!mbar_wait(&S->afull, na & 1, abortf, 1000000000ull, 64)) { ok = false; break; }
          ++na;
        }
        if (t.y < 0) {  // end of the item: the resident rows are free when these MMAs are done
          umma_commit(&S->aempty);
          continue;
        }
        const uint32_t b = acc & 1, aph = (acc >> 1) & 1;
        if (!mbar_wait(&S->tempty[b], aph ^ 1, abortf, 1000000000ull, 64)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tbase + b * 256;
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&S->full[stage], phase, abortf, 1000000000ull, 64)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = sbase + stage * TV_STAGE_BYTES;
#pragma unroll
          for (int ks = 0; ks < TV_KB / 16; ++ks) {
            const uint64_t bhi = umma_desc_sw64(st + ks * 32);
            const uint64_t blo = umma_desc_sw64(st + TV_SUB_BYTES + ks * 32);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const uint32_t at = abase + ((u * nkb + kb) * 2) * TV_SUB_BYTES + ks * 32;
              const uint64_t ahi = umma_desc_sw64(at);
              const uint64_t alo = umma_desc_sw64(at + TV_SUB_BYTES);
              umma_f16(d + u * TV_N, ahi, bhi, idesc, (kb | ks) != 0);
              umma_f16(d + u * TV_N, ahi, blo, idesc, 1);
              umma_f16(d + u * TV_N, alo, bhi, idesc, 1);
            }
          }
          umma_commit(&S->empty[stage]);
          if (++stage == (uint32_t)nst) { stage = 0; phase ^= 1; }
        }
        if (ok) umma_commit(&S->tfull[b]);
        ++acc;
      }
      if (!ok) {
        atomicMax(err, 2);
        *abortf = 1;
      }
      umma_commit(&S->done);
      volatile int dummy = 0;
      mbar_wait(&S->done, 0, &dummy, 200000000ull);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;
    const int q = warp & 3;            // TMEM lane quarter: rows 32q .. 32q + 31 of a row tile
    const int u = (ew >> 2) >> 1;      // row tile of the pair
    const int half = (ew >> 2) & 1;    // column half: 64 * half .. + 63
    const int r = u * 128 + 32 * q + lane;  // this lane's row of the item
    const int pbar = 2 + 4 * u + q;    // named barrier of the two warps sharing these 32 rows
    int* hist = scratch_all + ew * TV_SCR;
    float* sv = reinterpret_cast<float*>(hist);  // [16][32]: a chunk's screen values, column-major
    const int own0 = u * 128 + 32 * q + 16 * half;  // the 16 rows this warp compacts and publishes
    uint64_t* lists = work + (size_t)blockIdx.x * TV_ROWS * TC_CAPG;
    uint64_t* mylist = lists + (size_t)r * TC_CAPG + half * lcap;
    uint16_t* hp = heaps + ((size_t)r * 2 + half) * KH;         // this lane's (row, half) heap
    const uint16_t* hq = heaps + ((size_t)r * 2 + (half ^ 1)) * KH;  // the partner half's
    // the heaps' bound of row rr: each half holds its KH smallest, so the
    // 2 KH >= k1 values of both lie at or below the larger root; plus the slack
    auto heap_thr = [&](int rr) -> float {
      if (!KH) return INF;
      const uint32_t h0 = heaps[(size_t)rr * 2 * KH], h1 = heaps[((size_t)rr * 2 + 1) * KH];
      return tv_u16_float(max(h0, h1)) + S->rslack[rr][half];
    };
    const float slack = 2.0f * guard * __ldg(nmax);  // + 2 g |x|^2 of the row, at each item's start
    const float mul = corr ? -0.5f : -2.0f;
    uint32_t acc = 0;
    bool ok = true;
    int cur = -1, rp = 0, seg = 0, g = 0;
    float rc = INF;
    float rtn = INF;  // the row's shared threshold, loaded one tile ahead
    // The two warps of a pair meet at their named barrier twice per tile:
    // after the task read and the accumulator wait (whose outcomes are ANDed,
    // so both leave together), and after the appends (before compaction).
    for (uint32_t qs = 0;; ++qs) {
      const uint32_t slot = qs % TV_TQ, qph = (qs / TV_TQ) & 1;
      const bool got = mbar_wait(&S->tq_full[slot], qph, abortf);
      int2 task = make_int2(-1, -1);
      if (got) {
        const volatile int* tv = reinterpret_cast<volatile int*>(&S->task[slot]);
        task = make_int2(tv[0], tv[1]);
      }
      const uint32_t b = acc & 1, aph = (acc >> 1) & 1;
      bool ready = true;
      if (got && task.x >= 0 && task.y >= 0) ready = mbar_wait(&S->tfull[b], aph, abortf);
      tc_fence_after();
      __syncwarp();
      if (!bar_and(pbar, 64, got && ready)) { ok = false; break; }
      if (lane == 0) mbar_arrive(&S->tq_empty[slot]);
      if (task.x < 0) break;
      if (task.x != cur) {
        cur = task.x;
        const int2 rs = tv_item(cur, nseg, nitems / nseg, ncoltiles, near_first, diag, tdall);
        rp = rs.x;
        seg = rs.y;
        g = rp * TV_ROWS + r;
        const float rn = (g < nfit) ? __ldg(nf + g) : 0.0f;
        rc = (g >= nfit) ? INF : corr ? 0.5f - guard * rn : rn * (1.0f - guard);
        rtn = (g < nfit) ? __ldcg(rowthr + g) : INF;
        S->rslack[r][half] = slack + 2.0f * guard * rn;  // (each half's warp keeps its own copy)
      }
      if (task.y < 0) {
        // end of the item: publish the owned rows and clear their state
        for (int x = 0; x < 16; ++x) {
          const int rr = own0 + x;
          const int gg = rp * TV_ROWS + rr;
          if (gg < nfit && !pilot) {
            // (the published threshold goes to rowthr: the recheck's tau may
            // not exceed what any segment kept)
            const float tp = fminf(fminf(S->thr[rr], __ldcg(rowthr + gg)), heap_thr(rr));
            if (lane == 0 && KH) atomicMin(reinterpret_cast<int*>(rowthr + gg), __float_as_int(tp));
            const int64_t go = rperm ? (int64_t)__ldg(rperm + gg) : gg;
            tv_publish(lists + (size_t)rr * TC_CAPG, S->cnt2[rr][0], S->cnt2[rr][1], lcap, Kp, tp, hist,
                       candout + (go * nseg + seg) * Kp, cand_n + go * nseg + seg, lane, cperm);
          } else if (gg < nfit && S->cnt2[rr][0] + S->cnt2[rr][1] >= k1) {
            const int c = S->cnt2[rr][0] + S->cnt2[rr][1];
            float tk1 = INF;
            float t = warp_select_keep2(lists + (size_t)rr * TC_CAPG, S->cnt2[rr][0], lcap, S->cnt2[rr][1],
                                        c >= Kp ? Kp : 0, hist, lane, k1, &tk1);
            t = fminf(fminf(t, tk1 + S->rslack[rr][half]), heap_thr(rr));
            if (lane == 0) atomicMin(reinterpret_cast<int*>(rowthr + gg), __float_as_int(t));
          }
          if (lane == 0) {
            S->cnt2[rr][0] = 0;
            S->cnt2[rr][1] = 0;
            S->thr[rr] = INF;
          }
        }
        // both halves have read the owned rows' heaps: clear this lane's for
        // the next item (the next task's barrier orders the clears before
        // any read)
        bar_named(pbar, 64);
        for (int i = 0; i < KH; ++i) hp[i] = 0x7F80;
        __syncwarp();
        continue;
      }
      const int tile = task.y;
      int cnt = S->cnt2[r][half];
      // screen value = rc + colterm + mul * x.y; a pair passes below the
      // row's threshold (its own list's or another segment's)
      // (the shared threshold read for this tile was issued during the last
      // one: a value a tile old is only looser, and its L2 latency is hidden)
      const float lim0 = fminf(S->thr[r], rtn) - rc;
      if (g < nfit) rtn = __ldcg(rowthr + g);
      const float rsl = S->rslack[r][half];
      // the heaps' bound (read once per tile)
      const float lim = KH ? fminf(lim0, tv_u16_float(max((uint32_t)hp[0], (uint32_t)hq[0])) + rsl - rc) : lim0;
      const uint32_t tq = tbase + ((uint32_t)(q * 32) << 16) + b * 256 + u * TV_N + 64 * half;
      const int j0 = tile * TV_N + 64 * half;
      const float4* ct4 = reinterpret_cast<const float4*>(colterm + j0);
      // Four chunks of 16 columns; the next chunk's TMEM load is in flight
      // while this one is screened. A chunk's passes go into a per-lane bit
      // mask (no branch per pair) and its values into shared memory; only if
      // some lane has a pass does the warp run the append loop, over the set
      // bits of each lane's mask.
      uint32_t ga[16], gb[16];
      tmem_ld16(tq, ga);
      tmem_wait_ld();
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        uint32_t* cur = (cc & 1) ? gb : ga;
        uint32_t* nxt = (cc & 1) ? ga : gb;
        if (cc < 3) tmem_ld16(tq + 16 * (cc + 1), nxt);
        float4 c4[4];
#pragma unroll
        for (int t4 = 0; t4 < 4; ++t4) c4[t4] = __ldg(ct4 + cc * 4 + t4);
        // four independent mask chains; only passing values are parked
        uint32_t m4[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int t4 = 0; t4 < 4; ++t4) {
          const float cv[4] = {c4[t4].x, c4[t4].y, c4[t4].z, c4[t4].w};
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const float v = fmaf(mul, __uint_as_float(cur[4 * t4 + t]), cv[t]);
            if (v < lim) {
              sv[(4 * t4 + t) * 32 + lane] = v;
              m4[t4] |= 1u << (4 * t4 + t);
            }
          }
        }
        uint32_t mask = (m4[0] | m4[1]) | (m4[2] | m4[3]);
        if (__any_sync(0xffffffffu, mask != 0u)) {
          while (mask) {
            const int t = __ffs(mask) - 1;
            mask &= mask - 1;
            const float bv = fmaxf(sv[t * 32 + lane] + rc, 0.0f);
            if (cnt < lcap) mylist[cnt] = mds_pack_key(bv, j0 + 16 * cc + t);
            ++cnt;
            if (KH) tv_heap_push(hp, KH, tv_u16_up(bv));
          }
        }
        __syncwarp();
        if (cc < 3) tmem_wait_ld();
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&S->tempty[b]);
      ++acc;
      if (cnt > lcap) atomicMax(err, 4);  // cannot happen: compaction keeps room for a tile
      S->cnt2[r][half] = min(cnt, lcap);
      bar_named(pbar, 64);  // both halves of these rows are appended
      // compaction of the owned rows whose regions near full (or first fill):
      // lane x < 16 tests row own0 + x, and the warp visits only the rows
      // that need it (testing the 16 rows one after another cost ~5,000
      // cycles per tile in shared-memory round trips)
      unsigned todo;
      {
        const int rr = own0 + (lane & 15);
        const int c0 = S->cnt2[rr][0], c1 = S->cnt2[rr][1];
        // a region near full: cut both back to the K' best
        const bool cutl = c0 + c1 > Kp && (c0 > lcap - 64 || c1 > lcap - 64);
        // the row's first own threshold comes from its k1-th key as soon as
        // those arrive (a rank search that moves no key): tighter than the
        // shared one, it cuts appends. (Refreshing it after every k1 further
        // appends was measured slower: the searches cost more than the
        // appends they save.) With the heaps on, they give that threshold
        // without a search.
        const bool firstl = !KH && S->thr[rr] == INF && c0 + c1 >= k1;
        todo = __ballot_sync(0xffffffffu, lane < 16 && rp * TV_ROWS + rr < nfit && (cutl || firstl));
      }
      while (todo) {
        const int x = __ffs(todo) - 1;
        todo &= todo - 1;
        const int rr = own0 + x;
        const int gg = rp * TV_ROWS + rr;
        const int c0 = S->cnt2[rr][0], c1 = S->cnt2[rr][1];
        const bool cut = c0 + c1 > Kp && (c0 > lcap - 64 || c1 > lcap - 64);
        float tk1 = INF;
        float t = warp_select_keep2(lists + (size_t)rr * TC_CAPG, c0, lcap, c1, cut ? Kp : 0, hist, lane, k1,
                                    &tk1);
        t = fminf(fminf(t, tk1 + S->rslack[rr][half]), heap_thr(rr));
        if (lane == 0) {
          if (cut) {
            S->cnt2[rr][0] = Kp;
            S->cnt2[rr][1] = 0;
          }
          S->thr[rr] = t;
          atomicMin(reinterpret_cast<int*>(rowthr + gg), __float_as_int(t));
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
    tmem_dealloc(tbase, 512);
  }
}

// Largest K' of the vector screen: after a compaction the first region of a
// row's list keeps room for one more tile's half (64 keys).
int tcv_max_kprime() { return TV_LCAP - TV_N / 2; }
// Largest padded dimension: the resident rows must fit in shared memory.
int tcv_max_dp() { return TV_MAX_DP; }

// Column segments per row pair tile: enough work items that the last wave of
// the dynamic schedule is short (about 16 items per SM), at most 8.
int tcv_choose_nseg(mds_ctx* ctx, int nfit, int nref) {
  const int nrp = (nfit + TV_ROWS - 1) / TV_ROWS, nct = (nref + TV_N - 1) / TV_N;
  int nseg = (16 * ctx->num_sms + nrp - 1) / nrp;
  return std::max(1, std::min({nseg, 8, nct}));
}

// The tensor-core screen of knn_data. Xf/Xr: FP32 vectors [n][Dp] (Dp a
// multiple of 32, at most TV_MAX_DP), nf/nr their squared norms. same: Xf is
// Xr (a set screened against itself; the visit starts at the diagonal).
// order: screen in locality order with tile skipping (vec_order.cu; the
// Euclidean and correlation metrics). Writes the candidate lists candout [nfit][nseg][Kp]
// (each unsorted), their sizes cand_n [nfit][nseg], and rowthr [nfit]: the
// threshold below which a row's pairs were kept (the bound of every pair left
// out when a row's lists hold fewer than K' in all). *tiles: the column tiles
// computed (TV_ROWS x TV_N pairs each), pilot pass included.
int launch_screen_tcv(mds_ctx* ctx, const float* Xf, const float* nf, int nfit, const float* Xr, const float* nr,
                      int nref, int Dp, bool corr, int Kp, int k, int nseg, bool same, bool order, uint64_t* candout,
                      int* cand_n, float* rowthr, long long* tiles) {
  if (Kp > tcv_max_kprime()) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "tensor-core vector screen: K' too large");
  if (Dp % TV_KB || Dp > TV_MAX_DP)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "tensor-core vector screen: padded dimension %d", Dp);
  const int ncoltiles = (nref + TV_N - 1) / TV_N;
  if (nseg < 1 || nseg > ncoltiles) return mds_fail(ctx, MDS_ERR_INTERNAL, "bad segment count %d", nseg);
  // (below 16 column tiles the order is not worth its launches)
  if (order && (Dp > vec_order_max_dp() || nref < 16 * TV_N)) order = false;
  cudaStream_t s = ctx->stream;
  const int rowsA = (nfit + TV_ROWS - 1) / TV_ROWS * TV_ROWS, rowsB = ncoltiles * TV_N;
  const int rowsS = std::max(rowsA, rowsB);
  const int nrp = rowsA / TV_ROWS;
  DevBuf A(ctx), B(ctx), work(ctx), err(ctx), terms(ctx), nmax(ctx), devn(ctx);
  DevBuf cent(ctx), permr(ctx), permf(ctx), nrs(ctx), nfs(ctx), dlo(ctx), tdseg(ctx), tdall(ctx), rts(ctx);
  MDS_TRY(terms.alloc(ctx, sizeof(float) * (size_t)rowsS));
  MDS_TRY(nmax.alloc(ctx, sizeof(float)));
  MDS_CUDA(ctx, cudaMemsetAsync(nmax.p, 0, sizeof(float), s));
  MDS_TRY(devn.alloc(ctx, sizeof(unsigned)));
  MDS_CUDA(ctx, cudaMemsetAsync(devn.p, 0, sizeof(unsigned), s));
  const int* pr = nullptr;
  const int* pf = nullptr;
  if (order) {
    MDS_TRY(cent.alloc(ctx, sizeof(float) * 16 * (size_t)Dp));
    MDS_TRY(permr.alloc(ctx, sizeof(int) * (size_t)nref));
    MDS_TRY(nrs.alloc(ctx, sizeof(float) * (size_t)nref));
    MDS_TRY(vec_order(ctx, Xr, nref, Dp, cent.as<float>(), true, permr.as<int>()));
    pr = permr.as<int>();
    if (same) {
      pf = pr;
    } else {
      MDS_TRY(permf.alloc(ctx, sizeof(int) * (size_t)nfit));
      MDS_TRY(nfs.alloc(ctx, sizeof(float) * (size_t)nfit));
      MDS_TRY(vec_order(ctx, Xf, nfit, Dp, cent.as<float>(), false, permf.as<int>()));
      pf = permf.as<int>();
    }
  }
  // list regions: a compaction is due once a region holds more than
  // lcap - 64 keys (room for one tile's half); lcap - 64 - K' appends
  // between compactions keep them rare
  const int lcap = TV_LCAP;
  auto split = [&](const float* X, const float* nrm, int n, int rows, DevBuf& out, float* t, const int* perm,
                   float* nsorted) -> int {
    MDS_TRY(out.alloc(ctx, sizeof(__nv_bfloat16) * 2 * (size_t)Dp * rows));
    const int64_t total = (int64_t)rows * Dp;
    const int grid = (int)std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 16);
    ctx->stats.launches++;
    k_vec_split<<<grid, 256, 0, s>>>(X, n, Dp, rows, out.as<__nv_bfloat16>(), nrm, MDS_GUARD_TC, corr ? 1 : 0, t,
                                     t ? nmax.as<float>() : nullptr, perm, nsorted,
                                     (order && corr) ? devn.as<unsigned>() : nullptr);
    MDS_CUDA(ctx, cudaGetLastError());
    return MDS_OK;
  };
  const void* pA;
  const float* nfk = nf;  // row norms in the screen's row order
  if (same) {  // one split array serves both roles (rows padded to the larger tiling)
    MDS_TRY(split(Xr, nr, nref, rowsS, B, terms.as<float>(), pr, order ? nrs.as<float>() : nullptr));
    pA = B.p;
    if (order) nfk = nrs.as<float>();
  } else {
    MDS_TRY(split(Xr, nr, nref, rowsB, B, terms.as<float>(), pr, nullptr));
    MDS_TRY(split(Xf, nf, nfit, rowsA, A, nullptr, pf, order ? nfs.as<float>() : nullptr));
    pA = A.p;
    if (order) nfk = nfs.as<float>();
  }
  float* rt = rowthr;  // thresholds in the screen's row order
  if (order) {
    MDS_TRY(dlo.alloc(ctx, sizeof(float) * (size_t)nrp * ncoltiles));
    if (!same) {
      MDS_TRY(tdseg.alloc(ctx, sizeof(int) * (size_t)nrp * nseg));
      MDS_TRY(tdall.alloc(ctx, sizeof(int) * (size_t)nrp));
    }
    MDS_TRY(rts.alloc(ctx, sizeof(float) * (size_t)nfit));
    rt = rts.as<float>();
    MDS_CUDA(ctx, cudaMemsetAsync(rt, 0x7f, sizeof(float) * (size_t)nfit, s));
    // the bounds, with each row's threshold seeded from its k1-th distance to
    // its start tile's members (that tile is screened first, without a storm
    // of appends under no threshold); the seeds also let the bounds skip the
    // exact refinement of tiles the coarse bound already excludes
    MDS_TRY(vec_tile_bounds(ctx, Xr, pr, nref, Xf, pf, nfit, Dp, TV_N, nmax.as<float>(), dlo.as<float>(), nseg,
                            same ? nullptr : tdseg.as<int>(), same ? nullptr : tdall.as<int>(), k + 1, rt,
                            corr ? devn.as<unsigned>() : nullptr));
  } else {
    MDS_CUDA(ctx, cudaMemsetAsync(rt, 0x7f, sizeof(float) * (size_t)nfit, s));
  }
  CUtensorMap mA, mB;
  MDS_TRY(encode_map(ctx, &mA, pA, same ? rowsS : rowsA, Dp, 128, MDS_PREC_BF16X3));
  MDS_TRY(encode_map(ctx, &mB, B.p, same ? rowsS : rowsB, Dp, TV_N, MDS_PREC_BF16X3));
  const int nitems = nrp * nseg;
  const int grid = std::min(nitems, ctx->num_sms);
  MDS_TRY(work.alloc(ctx, sizeof(uint64_t) * (size_t)grid * TV_ROWS * TC_CAPG));
  MDS_TRY(err.alloc(ctx, 4 * sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(err.p, 0, 4 * sizeof(int), s));
  const int nst = (Dp <= 64) ? 4 : (Dp <= 96 ? 3 : 2);
  static bool attr_done = false;
  static size_t attr_limit = 0;
  MDS_TRY(mds_allow_dyn_smem(ctx, k_screen_tcv, &attr_done, &attr_limit));
  // threshold heaps of k1 entries per (row, column half) where they fit
  int KH = (k + 1 <= TV_KHMAX) ? (k + 2) / 2 : 0;
  if (KH && tv_smem_bytes(Dp, nst, KH) > attr_limit) KH = 0;
  const size_t smem = tv_smem_bytes(Dp, nst, KH);
  if (smem > attr_limit)
    return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "vector screen needs %zu bytes of shared memory", smem);
  const uint32_t idesc = umma_idesc_f16(128, TV_N, 1);
  const float* pdlo = order ? dlo.as<float>() : nullptr;
  const int* ptdseg = (order && !same) ? tdseg.as<int>() : nullptr;
  const int* ptdall = (order && !same) ? tdall.as<int>() : nullptr;
  // pilot pass (input order): seed every row's threshold from TV_PILOT
  // column tiles, so the main pass appends few pairs from its first tile on.
  // In locality order the near segments come first instead (tv_item).
  if (!order && ncoltiles >= 4 * TV_PILOT) {
    ctx->stats.launches++;
    k_screen_tcv<<<std::min(nrp, ctx->num_sms), TV_THREADS, smem, s>>>(
        mA, mB, nfk, terms.as<float>(), nfit, nref, Dp, nst, corr ? 1 : 0, MDS_GUARD_TC, idesc, Kp, 1, nrp,
        same ? 1 : 0, TV_PILOT, rt, work.as<uint64_t>(), candout, cand_n, err.as<int>(), lcap, k + 1,
        nmax.as<float>(), nullptr, nullptr, nullptr, 0, nullptr, nullptr, KH, nullptr);
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaMemsetAsync(err.as<int>() + 1, 0, sizeof(int), s));
  }
  ctx->stats.launches++;
  k_screen_tcv<<<grid, TV_THREADS, smem, s>>>(mA, mB, nfk, terms.as<float>(), nfit, nref, Dp, nst, corr ? 1 : 0,
                                              MDS_GUARD_TC, idesc, Kp, nseg, nitems, same ? 1 : 0, 0, rt,
                                              work.as<uint64_t>(), candout, cand_n, err.as<int>(), lcap, k + 1,
                                              nmax.as<float>(), pdlo, ptdseg, ptdall, order ? 1 : 0,
                                              pr ? pf : nullptr, pr, KH,
                                              (order && corr) ? devn.as<unsigned>() : nullptr);
  MDS_CUDA(ctx, cudaGetLastError());
  if (order) MDS_TRY(vec_unsort(ctx, rt, pf, nfit, rowthr));
  int herr[3] = {0, 0, 0};
  MDS_CUDA(ctx, cudaMemcpyAsync(herr, err.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  if (herr[0])
    return mds_fail(ctx, herr[0] == 4 ? MDS_ERR_INTERNAL : MDS_ERR_TIMEOUT,
                    "tensor-core vector screen failed (code %d)", herr[0]);
  if (tiles) *tiles = herr[2];
  return MDS_OK;
}
