/*
 * mdsgpu.h -- C ABI of libmdsgpu, the GB300 (sm_103a) implementation of the
 * MDSCTK 1.2.5 hot path: all-pairs minimum-RMSD kNN (knn_rms), vector kNN
 * (knn_data), symmetric / general sparse assembly (make_sysparse,
 * make_gesparse) and the sparse spectral eigensolve (decomp_sparse,
 * decomp_sparse_nystrom).
 *
 * The reference exposes these steps only as command-line tools over binary
 * files; every entry point below replaces the compute core of one tool and
 * keeps its argument meaning, output layout and ordering. The drop-in tools
 * (same flags, same files) in mdsctk_gb300/csrc/tools/ call these entry
 * points.
 *
 * Conventions:
 *  - Plain pointers and sizes only. Host pointers unless MDS_DEVICE_IO is set,
 *    in which case every array argument is a device pointer on the
 *    context's device.
 *  - Every function returns MDS_OK (0) or a negative MDS_ERR_* code; the
 *    message is in mds_last_error(ctx). No exceptions or exit() cross the ABI.
 *  - The caller owns every input and output buffer; the context owns all
 *    device scratch memory it allocates and frees it before returning.
 *  - A context serialises its calls on one CUDA stream; use one context per
 *    host thread.
 */
#ifndef MDSGPU_H
#define MDSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDS_OK 0
#define MDS_ERR_ARG (-1)         /* invalid argument (sizes, k, flags) */
#define MDS_ERR_CUDA (-2)        /* CUDA runtime / launch failure */
#define MDS_ERR_NOMEM (-3)       /* device allocation or HBM budget */
#define MDS_ERR_UNSUPPORTED (-4) /* shape outside a kernel's limits */
#define MDS_ERR_TIMEOUT (-5)     /* a bounded device wait gave up */
#define MDS_ERR_INTERNAL (-6)

/* flags */
#define MDS_NOFIT 0x1u        /* knn_rms -n true: RMSD without superposition */
#define MDS_FULL 0x2u         /* -s false: write full distance rows, no sort */
#define MDS_DEVICE_IO 0x4u    /* array arguments are device pointers */
#define MDS_CORRELATION 0x8u  /* knn_data -c: correlation distance */
#define MDS_PREC_FP32 0x00u   /* candidate screen on FP32 CUDA cores */
#define MDS_PREC_BF16X3 0x10u /* candidate screen on tcgen05, split BF16 (3 products) */
#define MDS_PREC_FP16X3 0x20u /* candidate screen on tcgen05, split FP16 (3 products) */
#define MDS_PREC_MASK 0xF0u

typedef struct mds_ctx mds_ctx;

/* Statistics of the last kNN call on a context. */
typedef struct mds_knn_stats {
  double prep_ms;      /* centring and superposition onto the template */
  double screen_ms;    /* all-pairs candidate screen with fused top-k */
  double recheck_ms;   /* candidate merge, exact recheck, output */
  double total_ms;     /* whole call, including host<->device copies */
  long long pairs;     /* N_fit * N_ref */
  int kprime;          /* candidates kept per row in the first pass */
  int rows_flagged;    /* rows whose guard failed in the first pass */
  int passes;          /* screen passes (1 + re-screens of flagged rows) */
  int screen_launches; /* kernel launches of the screen */
} mds_knn_stats;

/* Library version string. */
const char* mds_version(void);

/* Create a context on `device`. hbm_budget: maximum device bytes the context
 * may hold at once (0 = no limit). */
int mds_create(int device, size_t hbm_budget, mds_ctx** out);
int mds_destroy(mds_ctx* ctx);
const char* mds_last_error(const mds_ctx* ctx);
int mds_get_knn_stats(const mds_ctx* ctx, mds_knn_stats* out);

/*
 * knn_rms: for each fit frame, the k nearest reference frames by minimum
 * mass-weighted RMSD after optimal superposition.
 * Replaces knn_rms.cpp:38-41 (distance = do_fit + rmsdev x 10) and the row
 * loop knn_rms.cpp:186-293 (reset_x centring, blocks, permutation::sort(k+1),
 * position-0 drop, row-major writes).
 *   ref_xyz  [n_ref][natoms][3] float, nm, uncentred (as read from the file)
 *   fit_xyz  [n_fit][natoms][3] float, or NULL for fit = ref
 *   mass     [natoms] float
 *   k        neighbours per row; clamped to n_ref-1 as knn_rms.cpp:224-225
 *   out_d    [n_fit][k] double, Angstrom (RMSD x 10), ascending; with
 *            MDS_FULL: [n_fit][n_ref] unsorted distances
 *   out_i    [n_fit][k] int32 reference indices (0-based); with MDS_FULL:
 *            [n_fit][n_ref] = 0..n_ref-1
 *   k_used   optional: receives the clamped k
 * Entries [1..k] of the k+1 nearest are written, as the reference does.
 */
int mds_knn_rms(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz, int n_fit,
                int natoms, const float* mass, int k, unsigned flags, double* out_d,
                int32_t* out_i, int* k_used);

/*
 * knn_data: k nearest reference vectors by Euclidean distance
 * (euclidean_distance, mdsctk.cpp:330-335) or, with MDS_CORRELATION, by
 * correlation distance (mdsctk.cpp:337-360). Replaces knn_data.cpp:176-250.
 *   ref [n_ref][dim] double, fit [n_fit][dim] double or NULL for fit = ref.
 * Distances are recomputed in FP64 in the reference's summation order, so
 * written values are bit-identical to the reference's.
 */
int mds_knn_data(mds_ctx* ctx, const double* ref, int n_ref, const double* fit, int n_fit,
                 int dim, int k, unsigned flags, double* out_d, int32_t* out_i, int* k_used);

#ifdef __cplusplus
}
#endif

#endif /* MDSGPU_H */
