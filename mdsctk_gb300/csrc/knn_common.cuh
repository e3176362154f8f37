// knn_common.cuh -- plan, sorting helpers and cross-file declarations of the
// kNN pipelines (knn_rms.cu, knn_rms_tc.cu, knn_data.cu, knn_api.cu).
#pragma once

#include <cuda.h>

#include <vector>

#include "mds_common.cuh"

// Screen guards: the lower bound of RMSD^2 is the screen value minus
// c * (|a_i|^2 + |a_j|^2), a = deviation from the template. c covers the
// rounding of the screen's Gram (FP32 FMA chains, or split BF16/FP16
// products accumulated in FP32 by the tensor cores). Measured over the
// 256 nearest candidates of sampled rows (20,000 x 1,000-atom trajectory and
// 50,000 x 304-atom landmarks against off-trajectory queries), the largest
// over-estimate per unit of |a_i|^2 + |a_j|^2 was 1.3e-6 (FP32), 6.1e-6
// (BF16x3) and 9.6e-6 (FP16x3): the guards below are 12x and 6x above them.
#define MDS_GUARD_FP32 (1.0f / 65536.0f)
#define MDS_GUARD_TC (1.0f / 16384.0f)

struct KnnRmsPlan {
  int nref = 0, nfit = 0, natoms = 0;
  int Ap = 0;      // natoms rounded up to 64 (zero-padded atoms)
  int k = 0;       // clamped k
  int kprime = 0;  // candidates kept per row by the screen
  int nofit = 0, full = 0;
  int noskip = 0;  // MDS_NO_SKIP: the tensor-core screen computes every tile
  unsigned prec = MDS_PREC_FP32;
  float guard_fp32 = 0.f;  // lower-bound margin per unit of |a_i|^2+|a_j|^2
  float guard_tc = 0.f;
  // diagnostic mode (mds_knn_rms_screen): stop after the screen, one column
  // segment, and copy the candidate lists to these host buffers
  uint64_t* screen_keys = nullptr;  // [nfit][kprime]
  int* screen_counts = nullptr;     // [nfit]
  // diagnostic mode (mds_knn_rms_superpose): stop after the superposition
  // onto the template and copy the reference set's deviations and records
  float* prep_dev = nullptr;  // [nref][3][Ap]
  float* prep_rec = nullptr;  // [nref][16]
  // host copies of the frames: when set, the device frame buffers passed to
  // knn_rms_run are filled here in chunks on the copy streams, and each chunk
  // is superposed as soon as it has landed
  const float* href = nullptr;
  const float* hfit = nullptr;
};

// Split hi/lo tensor-core operands of one frame set (knn_rms_tc.cu).
struct TcOperands {
  DevBuf A, B;     // row-tile (fit role) and column-tile (reference role) layouts
  int n = 0;       // frames
  int rowsA = 0, rowsB = 0;
  int K = 0;       // padded atoms per split part (row length is 2K: hi | lo)
};

__device__ __forceinline__ void warp_bitonic_sort(uint64_t* a, int n, int P2, int lane) {
  for (int x = n + lane; x < P2; x += 32) a[x] = MDS_KEY_INF;
  __syncwarp();
  for (int k = 2; k <= P2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P2; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint64_t x = a[i], y = a[ixj];
          bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
}

// All threads of the block; P2 a power of two; a[] fully initialised.
__device__ __forceinline__ void block_bitonic_sort(uint64_t* a, int P2) {
  for (int k = 2; k <= P2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint64_t x = a[i], y = a[ixj];
          bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncthreads();
    }
}

// The correlation metric's squared distance (1 - r) / 2 of two standardised
// vectors is |z_x - z_y|^2 / 4 of their FP32 operands within this margin:
// half the largest | |z|^2 - 1 | of the FP32 norms (devn, the float's bits),
// the norms' summation error (< Dp 2^-24), and the operands' rounding to
// FP32 (< 2^-24 |z| per vector).
__device__ __forceinline__ float corr_margin(const unsigned* devn, int Dp) {
  return 0.5f * __uint_as_float(__ldg(devn)) + 1e-7f * (float)Dp + 1e-6f;
}

__host__ __device__ static inline int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

int knn_rms_run(mds_ctx* ctx, KnnRmsPlan& pl, const float* draw_ref, const float* draw_fit,
                const float* hmass, double* dout_d, int* dout_i);

// pieces of the knn_rms pipeline (knn_rms.cu), reused by the serving loop
int launch_center(mds_ctx* ctx, const float* draw, int n, int natoms, int Ap, const float* dmass,
                  const float* dswn, float tm, float* Y, double* E);
// Centring + superposition of n raw frames (three kernels, no scratch
// buffer): deviations and records only (knn_rms.cu).
// Uhl (optional): the frames' U = sum a mu^T as double-float pairs [n][18],
// which the recheck needs for the reference frames.
int launch_prep(mds_ctx* ctx, const float* draw, int n, int natoms, int Ap, const float* dmass, const float* dswn,
                float tm, const float* dmu, const double* dM0, int nofit, float* A, float* R, float* Uhl = nullptr,
                int* bad = nullptr, int fbase = 0);
int build_template(mds_ctx* ctx, const float* dY0, int Ap, int natoms, bool nofit, std::vector<double>& mu,
                   double M0[9]);
// Frames per row tile (40: 128 MMA rows, 10 frames per 32-lane quarter) and
// per column tile (80: 240 MMA columns) of the tensor-core screen; the tile
// skipping data (pivots, radii, row-tile bounds) is laid out on these tiles.
#define TC_FR_M 40
#define TC_FR_N 80

// Optional parts of the FP32 screen (k_screen_fp32, knn_rms.cu): tile
// skipping with the tensor-core screen's row-tile pivots (pivlb [nR][nfit]
// lower bounds of RMSD to the pivots, prad [2 nC] radii of the 80-frame
// column tiles, rowlo [nR][nC]), shared row thresholds, thresholds from the
// (k+1)-th bound, outward column order, and the dense pivot pass.
struct Fp32ScreenExtra {
  const float* pivlb = nullptr;
  const float* prad = nullptr;
  const float* rowlo = nullptr;
  int nR = 0, nC = 0, nfit = 0;
  float* rowthr = nullptr;
  const float* nmax = nullptr;
  int k1 = 0;
  int diag = 0;
  float* dense = nullptr;  // [nref][nrows]
  unsigned long long* ntiles = nullptr;  // tiles computed (32 x 64 frames each)
};
int launch_screen_fp32(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Af, const float* Ar, const float* recf,
                       const float* recr, int nrows, const int* rowlist, int Kp, int nseg, uint64_t* cand,
                       int* cand_n, const Fp32ScreenExtra* extra = nullptr);
// Exact recheck from the superposed deviations (Af/Ar [n][3][Ap]) and the
// template mu [3][Ap] (knn_rms.cu).
// Ur: the reference frames' U as written by launch_prep (unused with nofit).
// Audit of the screen's bounds by the recheck (mode 0): the fit and
// reference records (|a|^2 in entry 15), the guard coefficient of the screen
// that produced the candidates, and four device counters: candidates
// rechecked, bounds above their exact value, the largest screen error per
// unit of |a_i|^2 + |a_j|^2 (float bits), rows flagged for a violation.
struct RecheckAudit {
  const float* recf = nullptr;
  const float* recr = nullptr;
  float guard = 0.f;
  unsigned long long* counters = nullptr;
};
int launch_recheck(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Af, const float* Ar, const float* mu,
                   const float* Ur, int nrows, const int* rowlist, int mode, const uint64_t* cand,
                   const int* cand_n, int nseg, int segstride, int Kp, int k, double* out_d, int* out_i,
                   int* flagged, int* nflag, const float* rowthr = nullptr, const RecheckAudit* audit = nullptr,
                   int cand_by_row = 0);

int choose_nseg_fp32(int nfit, int num_sms, int nref);

// Candidates wanted per row before rounding: k+33, 2(k+1), and with the
// tensor-core screen 4(k+1) up to 256 (its thresholds follow the (k+1)-th
// bound, so a deeper list only helps the guard check of crowded rows).
inline int tc_kprime_want(int k, bool tc) {
  int w = std::max(k + 1 + 32, 2 * (k + 1));
  if (tc) w = std::max(w, std::min(4 * (k + 1), 256));
  return w;
}

// tensor-core screen (knn_rms_tc.cu)
int tc_prepare(mds_ctx* ctx, const KnnRmsPlan& pl, const float* dev, int n, TcOperands& op, int layout);
int tc_seg_stride();
int tc_choose_nseg(mds_ctx* ctx, const KnnRmsPlan& pl, int nfit);
// 2-D tensor map of a split hi|lo operand: rows x (2 * half) 16-bit values,
// boxes of 32 x boxrows, 64-byte swizzle (knn_rms_tc.cu).
int encode_map(mds_ctx* ctx, CUtensorMap* map, const void* ptr, int rows, int half, int boxrows, unsigned prec);

// tensor-core screen of knn_data (knn_data_tc.cu)
int tcv_max_kprime();
int tcv_max_dp();
int tcv_choose_nseg(mds_ctx* ctx, int nfit, int nref);
int launch_screen_tcv(mds_ctx* ctx, const float* Xf, const float* nf, int nfit, const float* Xr, const float* nr,
                      int nref, int Dp, bool corr, int Kp, int k, int nseg, bool same, bool order, uint64_t* candout,
                      int* cand_n, float* rowthr, long long* tiles);

// locality order and tile bounds of a vector set (vec_order.cu)
int vec_order_max_dp();
int vec_order(mds_ctx* ctx, const float* X, int n, int Dp, float* cent, bool fit, int* perm);
int vec_tile_bounds(mds_ctx* ctx, const float* Xr, const int* permr, int nref, const float* Xf, const int* permf,
                    int nfit, int Dp, int tile, const float* nmax, float* dlo, int nseg, int* tdseg, int* tdall,
                    int k1, float* rowthr, const unsigned* devn);
int vec_seed_rows(mds_ctx* ctx, const float* Xr, const int* permr, int nref, const float* Xf, const int* permf,
                  int nfit, int Dp, const int* tdall, int k1, const float* nmax, float* rowthr,
                  const unsigned* devn);
int vec_unsort(mds_ctx* ctx, const float* src, const int* perm, int n, float* dst);

// Tile skipping data of the tensor-core screen (knn_rms_tc.cu): lower
// bounds of RMSD from every fit frame to the pivot of every column tile
// (pivlb [ncoltiles][nfit]) and the tiles' radii (prad [ncoltiles]).
struct TcSkip {
  const float* pivlb = nullptr;
  const float* prad = nullptr;
  const float* rowlo = nullptr;  // [nrowtiles][ncoltiles] row-tile bounds, or null
  int piv2 = 0;                  // pivots are the row tiles' (two per column tile)
  const int* far_perm = nullptr; // order of the non-diagonal items, or null
};
// The pivots of a reference set (their deviations, records and split
// operands) and the radii: the middle frame of every column tile (nP = nC),
// or, for a set screened against itself (rowpiv), of every row tile
// (nP = row tiles, rad = two radii per column tile, rrad = the row tiles').
struct TcPivots {
  DevBuf A, R, rad, rrad, idx;
  TcOperands tc;
  std::vector<int> hidx;  // the pivots' frame indices
  int nC = 0, nP = 0;
  bool rowpiv = false;
};
int tc_skip_pivots(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Ar, const float* Rr, TcPivots& pv,
                   bool rowpiv = false);
// The same in steps, for frames prepared chunk by chunk: indices and buffers
// (radii zeroed); the split pivot operand once pv.A / pv.R hold the pivots'
// deviations and records; the radii of the row tiles of frames [f0, f1)
// (row-tile pivots; f0 a multiple of a column tile).
int tc_pivots_begin(mds_ctx* ctx, const KnnRmsPlan& pl, TcPivots& pv, bool rowpiv);
int tc_pivots_operand(mds_ctx* ctx, const KnnRmsPlan& pl, TcPivots& pv);
int tc_pivots_radii(mds_ctx* ctx, const KnnRmsPlan& pl, const float* Ar, TcPivots& pv, int f0, int f1);
int tc_skip_rowlo(mds_ctx* ctx, const TcPivots& pv, const float* lb, int n, float* rowlo);
// Order of the non-diagonal work items of a self screen with nseg segments,
// estimated heaviest first (work: 3 * 1024 + row tiles * (nseg - 1) ints;
// perm: row tiles * (nseg - 1) ints).
int tc_far_order(mds_ctx* ctx, const TcPivots& pv, const float* lb, const float* rowlo, int n, int nseg,
                 int* work, int* perm);
int tc_skip_bounds(mds_ctx* ctx, const KnnRmsPlan& pl, const TcOperands& fit, const float* recf, int nfit,
                   const TcPivots& pv, float* lb, int* derr = nullptr, int f0 = 0, int f1 = 0);
// rt0 / nrt_items: the row tiles [rt0, rt0 + nrt_items) only (dense mode;
// nrt_items < 0: every row tile)
int launch_screen_tc(mds_ctx* ctx, const KnnRmsPlan& pl, const TcOperands& fit, const TcOperands& ref,
                     const float* recf, const float* recr, int nfit, int Kp, int nseg, uint64_t* cand,
                     int* cand_n, int* derr = nullptr, const TcSkip* skip = nullptr,
                     float* dense = nullptr, float* rowthr = nullptr, const float* nmax = nullptr,
                     unsigned long long* ntiles = nullptr, int rt0 = 0, int nrt_items = -1);
// Split operands in steps: the buffer for n frames, then the rows of frames
// [f0, f1) (f0 a multiple of a column tile; f1 too unless it is n).
int tc_alloc(mds_ctx* ctx, const KnnRmsPlan& pl, int n, TcOperands& op, int layout);
int tc_prepare_range(mds_ctx* ctx, const KnnRmsPlan& pl, const float* dev, int n, TcOperands& op, int layout,
                     int f0, int f1);
// *out = the largest |a|^2 over the records rec[n] (a device float).
int tc_rec_nmax(mds_ctx* ctx, const float* rec, int n, float* out);
