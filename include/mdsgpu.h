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
#define MDS_NO_SKIP 0x100u    /* knn_rms and knn_data, tensor-core screen:
                                 compute every tile (no triangle-inequality tile
                                 skipping; knn_data also keeps the input order).
                                 Same results; for timing the screens like for
                                 like */

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
  int launches;        /* all kernel launches of the call */
  long long screen_pairs; /* pairs the first-pass screen computed: tiles not
                             skipped (40 x 80 frames each) plus the pivot pass */
  long long recheck_pairs; /* candidates the first-pass recheck computed exactly */
  int guard_violations;    /* rechecked candidates whose screen lower bound was
                              above their exact RMSD^2 (rows flagged; expected 0) */
  float screen_err_max;    /* largest screen error over the rechecked pairs,
                              (screen RMSD^2 - exact) / (|a_i|^2 + |a_j|^2): the
                              quantity the guard coefficient must exceed */
  float guard_coef;        /* guard coefficient of the first-pass screen */
  int rows_audit_flagged;  /* rows flagged because of a guard violation */
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
 * Fault injection for tests of the failure paths (no reference
 * counterpart: the reference's tools only return exit codes). Arms a fault
 * for the next call on ctx that reaches it; each fires once.
 *   MDS_INJECT_SCREEN_STALL: the next tensor-core screen launch withholds its
 *   end-of-work marker, so the kernel's bounded waits run out after about a
 *   second; the kernel then releases its resources and reports it, and the
 *   call returns MDS_ERR_TIMEOUT. The context stays usable.
 * what = 0 disarms.
 */
#define MDS_INJECT_SCREEN_STALL 0x1u
int mds_test_inject(mds_ctx* ctx, unsigned what);

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
 * Host frames are uploaded in chunks that overlap the superposition; from
 * page-locked (cudaHostAlloc / registered) memory the uploads run
 * asynchronously and, for a set against itself, the screen's operands and
 * pivot bounds are built chunk by chunk during the upload as well.
 */
int mds_knn_rms(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz, int n_fit,
                int natoms, const float* mass, int k, unsigned flags, double* out_d,
                int32_t* out_i, int* k_used);

/*
 * Diagnostic of the knn_rms candidate screen (no reference counterpart: the
 * reference computes every pair exactly). Runs centring, superposition onto
 * the template and the screen selected by the precision flag, and returns,
 * per fit frame, the `kprime` smallest screen keys in ascending order:
 * (float lower bound of RMSD^2 in nm^2, as its bit pattern) << 32 | index.
 *   keys [n_fit][kprime] uint64, counts [n_fit] (entries valid per row).
 */
int mds_knn_rms_screen(mds_ctx* ctx, const float* ref_xyz, int n_ref, const float* fit_xyz, int n_fit,
                       int natoms, const float* mass, int kprime, unsigned flags, uint64_t* keys,
                       int32_t* counts);

/*
 * Diagnostic of the superposition step of knn_rms (no reference
 * counterpart): every frame centred (reset_x), scaled by sqrt(mass/M) and
 * superposed onto the template (the first frame in its principal axes).
 *   dev [n_ref][3][Ap] float deviations a = R y - mu, Ap = natoms rounded
 *       up to 64 (padding zero); rec [n_ref][16] float screen records:
 *       M0+sym(U) (6), sym(U) (6), antisym(U) (3), |a|^2, with U = sum a mu^T.
 */
int mds_knn_rms_superpose(mds_ctx* ctx, const float* ref_xyz, int n_ref, int natoms, const float* mass,
                          unsigned flags, float* dev, float* rec);

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

/*
 * knn_data without device allocation. This entry point has no counterpart in
 * the reference. It is for callers that cannot allocate device memory where
 * they call, such as a plugin running inside another framework whose caching
 * allocator has reserved the device memory in full (a cudaMalloc there fails
 * or takes memory the host framework counts on). It computes what
 * mds_knn_data computes (same outputs), takes DEVICE pointers for every
 * array, and keeps all of its scratch in one fixed 32 MiB array inside the
 * library, so it calls no cudaMalloc/cudaFree and no allocating library
 * routine. Problems whose scratch would exceed 32 MiB (about n_fit * K' * 8
 * bytes of candidates, K' = 1.5(k+1) rounded up to 32 and at most 192, plus
 * n * dim * 4 bytes of vectors) are rejected with MDS_ERR_UNSUPPORTED. When
 * K' < k + 17 every row is rechecked exactly, as mds_knn_data does.
 *   flags: 0 or MDS_CORRELATION (sorted output only).
 * The call synchronises ctx's stream before it returns and reads a device
 * count on the host to decide on a second pass, so it cannot be recorded
 * into a CUDA graph. The first call on a device also looks up the array's
 * device address (cudaGetSymbolAddress, once per device).
 * Calls share the array and it keeps the last call's contents: calls that
 * may overlap on the GPU (other contexts or threads) race and must be
 * serialised by the caller. The caller's current device is restored on
 * return. Every GPU that loads the library holds the 32 MiB until the
 * process exits.
 */
int mds_knn_data_noalloc(mds_ctx* ctx, const double* ref, int n_ref, const double* fit, int n_fit, int dim, int k,
                         unsigned flags, double* out_d, int32_t* out_i, int* k_used);

/*
 * knn_data_sparse: k nearest sparse vectors by euclidean_distance_sparse
 * (mdsctk.cpp:362-386). Replaces knn_data_sparse.cpp:176-260 (the reference
 * reads the vectors from an index file of [int n][int idx[n]] records and a
 * data file of [double val[n]] records; the tool knn_data_sparse does).
 *   ref: CSR rows ref_off[n_ref+1] (int64, ref_off[0] = 0), ref_idx, ref_val.
 *   fit: the same, or fit_off NULL for fit = ref.
 *   flags: 0, or MDS_FULL for the full row of distances in reference order
 *   (the reference's -s false; out_i then holds 0..n_ref-1).
 * Distances are the reference's FP64 walk, operation for operation, so the
 * written values are bit-identical to the reference's; indices of equal
 * distances are ordered by index (the reference leaves that order open).
 * Host buffers; k is clamped to n_ref - 1 and returned in k_used.
 */
int mds_knn_data_sparse(mds_ctx* ctx, const int64_t* ref_off, const int32_t* ref_idx, const double* ref_val,
                        int n_ref, const int64_t* fit_off, const int32_t* fit_idx, const double* fit_val, int n_fit,
                        int k, unsigned flags, double* out_d, int32_t* out_i, int* k_used);

/*
 * contact_profile: sparse binary contact maps (contact_profile.cpp:200-262).
 * For every frame of xyz [nframes][natoms][3] (float, nm) the atom pairs
 * (g1[i], g2[j]) (0-based atom indices) at distance * 10 < eps (Angstrom)
 * are contacts; a frame's vector holds the ascending grid indices i*n2 + j
 * of its contacts, each with value 1.0. Writes offsets[nframes+1] (int64,
 * offsets[0] = 0); with idx != NULL and idx_cap >= offsets[nframes] also the
 * indices (call first with idx = NULL to size the buffer). Contacts are
 * decided in the reference's arithmetic (float differences and squares, a
 * double sum, sqrt, times 10), so the sets are identical.
 */
int mds_contact_profile(mds_ctx* ctx, const float* xyz, int nframes, int natoms, const int32_t* g1, int n1,
                        const int32_t* g2, int n2, double eps, int64_t* offsets, int32_t* idx, int64_t idx_cap);

/*
 * GROMACS .xtc trajectories, the input format of knn_rms (read through
 * GROMACS in the reference: read_first_xtc / read_next_xtc,
 * knn_rms.cpp:155-203; XTC_file, mdsctk.cpp:217-267).
 *
 * mds_xtc_index walks the frame headers of an in-memory .xtc file (host
 * code, no context). With offsets == NULL it only counts: *nframes frames of
 * *natoms atoms. Otherwise offsets [max_frames] receives the byte offset of
 * every frame and, if room is left, the end offset after the last one
 * (pass max_frames >= nframes + 1). A truncated last frame is not counted
 * (read_next_xtc stops there). Returns MDS_ERR_ARG on a bad magic number or
 * a change of atom count.
 */
int mds_xtc_index(const unsigned char* buf, size_t len, int64_t* offsets, int max_frames, int* nframes,
                  int* natoms);

/*
 * mds_xtc_decode decodes nframes frames (offsets [nframes + 1] from
 * mds_xtc_index) on the GPU, one thread per frame, into xyz
 * [nframes][natoms][3] float nm, exactly as GROMACS decodes them
 * (int * (float)(1/precision)). buf is host memory; with MDS_DEVICE_IO, xyz
 * is a device pointer and the frames stay in HBM for mds_knn_rms. steps,
 * times [nframes] and boxes [nframes][9] are optional host outputs (NULL to
 * skip). A malformed frame returns MDS_ERR_ARG naming the frame.
 */
int mds_xtc_decode(mds_ctx* ctx, const unsigned char* buf, size_t len, const int64_t* offsets, int nframes,
                   int natoms, unsigned flags, float* xyz, int* steps, float* times, float* boxes);

/*
 * make_sysparse: kNN lists -> symmetric sparse matrix holding one strict
 * triangle of distances, CSC (column c holds rows r > c, ascending).
 * Replaces make_sysparse.cpp:225-329 (Berkeley-DB B-tree insertion with
 * compare_edge, mdsctk.cpp:567-577, put-overwrite, cursor walk split_edges,
 * mdsctk.cpp:580-604). Rows r = 0..n_rows-1 of dist/idx ([n_rows][maxk]),
 * first k entries of each row (-n, k <= maxk). For an edge listed by both
 * ends, the later row's value wins, as the later put does.
 *   pcol [n_rows+1], irow [cap], val [cap]; *nnz receives the count
 *   (cap >= n_rows * k always suffices).
 */
int mds_sysparse(mds_ctx* ctx, const double* dist, const int32_t* idx, int n_rows, int maxk, int k,
                 unsigned flags, int32_t* pcol, int32_t* irow, double* val, int64_t cap, int64_t* nnz);

/*
 * make_gesparse: kNN lists of queries against landmarks -> general CSC,
 * column = query row, rows = landmark indices ascending; with `symmetric`
 * (-s) also the transposed entry where it is absent at insertion time.
 * Replaces make_gesparse.cpp:246-335. cap >= n_rows * k * (symmetric ? 2 : 1).
 */
int mds_gesparse(mds_ctx* ctx, const double* dist, const int32_t* idx, int n_rows, int maxk, int k,
                 int symmetric, unsigned flags, int32_t* pcol, int32_t* irow, double* val, int64_t cap,
                 int64_t* nnz);

/*
 * decomp_sparse: Gaussian affinity exp(-d^2 / 2 sigma^2) of the stored
 * triangle, symmetric normalisation D^-1/2 W D^-1/2, and the nev largest
 * eigenpairs ('LA'). Replaces decomp_sparse.cpp:138-277 and its ARPACK
 * driver (dsaupd/dseupd, :185-237).
 *   n, pcol [n+1], irow [nnz], dist [nnz]: the .ssm matrix (CSC).
 *   ncv <= 0: min(10 nev + 1, n) as the reference; tol <= 0: machine
 *   epsilon (tol = 0 in the reference); maxiter <= 0: 100 nev.
 *   evals [nev] descending; evecs [nev][n] in the same order (unit norm,
 *   sign arbitrary as ARPACK's); resid [nev] = ||A z - lambda z|| / |lambda|
 *   (may be NULL); nconv receives the converged count (may be NULL).
 */
int mds_decomp_sparse(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow, const double* dist,
                      double sigma, int nev, int ncv, double tol, int maxiter, unsigned flags, double* evals,
                      double* evecs, double* resid, int* nconv);

/*
 * decomp_sparse_nystrom: decomp_sparse plus the Nystrom extension of the
 * eigenvectors to m out-of-sample queries: B = the .gsm matrix (CSC, column =
 * query, rows = landmarks) kernelised with the landmark degrees and its own
 * column sums, ext[x] = B^T (z_x / lambda_x). Replaces
 * decomp_sparse_nystrom.cpp:173-312. ext [nev][m].
 */
int mds_decomp_sparse_nystrom(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow, const double* dist,
                              int m, const int32_t* pcolB, const int32_t* irowB, const double* distB,
                              double sigma, int nev, int ncv, double tol, int maxiter, unsigned flags,
                              double* evals, double* evecs, double* ext, double* resid, int* nconv);

/*
 * auto_decomp_sparse: decomp_sparse with a sigma per landmark instead of one
 * sigma. Landmark x's list is its stored distances in neighbour-index order,
 * cut to the first k_sigma entries, then sorted; sigma_x = sum / k_sigma
 * (auto_decomp_sparse.cpp:153-168). perplexity > 0 (-K) replaces them by
 * entropic-affinity sigmas, the distribution over the k_sigma sorted
 * distances having perplexity K (mdsctk.cpp:388-565; agrees with the
 * reference to the root-finding tolerance, as the reference warm-starts each
 * landmark from the previous one). Affinity exp(-d^2 / (2 s_c s_r)) of the
 * stored entry's column c and row r (:180-182); the rest as decomp_sparse.
 * Replaces auto_decomp_sparse.cpp:135-258. sigmas [n] receives the sigmas
 * (may be NULL). k_sigma <= 4096; with perplexity, every landmark must hold
 * at least k_sigma >= ceil(K) distances (the reference reads past shorter
 * lists), else MDS_ERR_ARG.
 */
int mds_auto_decomp_sparse(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow, const double* dist,
                           int k_sigma, double perplexity, int nev, int ncv, double tol, int maxiter, unsigned flags,
                           double* evals, double* evecs, double* resid, int* nconv, double* sigmas);

/*
 * auto_decomp_sparse_nystrom: auto_decomp_sparse plus the Nystrom extension;
 * B's affinity uses the landmark's sigma twice, exp(-d^2 / (2 s_l s_l))
 * (auto_decomp_sparse_nystrom.cpp:171-173). The reference tool accepts -K
 * but never applies it (its perplexity switch is not set); its CLI here
 * passes perplexity 0 the same way. Replaces
 * auto_decomp_sparse_nystrom.cpp:140-285.
 */
int mds_auto_decomp_sparse_nystrom(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow,
                                   const double* dist, int m, const int32_t* pcolB, const int32_t* irowB,
                                   const double* distB, int k_sigma, double perplexity, int nev, int ncv, double tol,
                                   int maxiter, unsigned flags, double* evals, double* evecs, double* ext,
                                   double* resid, int* nconv, double* sigmas);

/*
 * Resident Nystrom serving (no single reference counterpart: it keeps on the
 * device what the file pipeline examples/cluster_rms_nystrom.bash:54-66
 * recomputes per run -- knn_rms on the landmarks, make_sysparse,
 * decomp_sparse_nystrom's eigenpairs and degrees -- and serves query frames:
 * knn_rms -f queries (nearest landmark dropped), make_gesparse and the
 * extension ext = B^T z / lambda, decomp_sparse_nystrom.cpp:181-219,301-312).
 * Requests are admitted continuously into batches (slots sized by the HBM
 * budget), each batch runs as a captured CUDA graph on its slot's stream.
 */
typedef struct mds_server mds_server;

typedef struct mds_server_config {
  int device;
  int k;                /* neighbours per frame (landmark graph and queries) */
  double sigma;         /* Gaussian kernel width, in the distance file's units (Angstrom) */
  int nev, ncv;         /* eigenpairs; ncv <= 0: min(10 nev + 1, n) */
  double tol;           /* <= 0: machine epsilon */
  int maxiter;          /* <= 0: 100 nev */
  unsigned flags;       /* MDS_PREC_*, MDS_NOFIT */
  int max_batch_frames; /* frames per batch (and per request); <= 0: 4096 */
  int slots;            /* concurrent batches (<= 0: 3), bounded by the HBM budget */
  size_t hbm_budget;    /* bytes for the slots; 0: half the free device memory */
  int use_graphs;       /* capture each batch size bucket in a CUDA graph */
} mds_server_config;

typedef struct mds_request_info {
  double queue_ms; /* submit -> admitted into a batch */
  double total_ms; /* submit -> results published */
  int batch;       /* batch id */
  int batch_frames;
} mds_request_info;

typedef struct mds_server_stats {
  int slots;
  long long slot_bytes;
  long long requests_submitted, requests_done, batches, frames;
  long long graph_launches, graphs_captured, rows_flagged;
  double model_knn_ms, model_decomp_ms;
  int model_nconv;
} mds_server_stats;

/* Build the landmark model from land_xyz [n][natoms][3] (nm) and start the
 * serving thread. */
int mds_server_create(const mds_server_config* cfg, const float* land_xyz, int n, int natoms, const float* mass,
                      mds_server** out);
int mds_server_destroy(mds_server* s);
const char* mds_server_last_error(const mds_server* s);
/* evals [nev] descending, evecs [nev][n] (may be NULL) of the landmark model */
int mds_server_model(mds_server* s, double* evals, double* evecs);
/* Queue m query frames [m][natoms][3] (copied); returns a ticket. */
int mds_server_submit(mds_server* s, const float* query_xyz, int m, int64_t* ticket);
/* Wait up to timeout_ms for a ticket: ext [nev][m] (eigenvector x, query q),
 * knn_d [m][k] (Angstrom), knn_i [m][k] (landmark ids); any may be NULL.
 * MDS_ERR_TIMEOUT if it is not done yet (the ticket stays valid). */
int mds_server_wait(mds_server* s, int64_t ticket, int timeout_ms, double* ext, double* knn_d, int32_t* knn_i,
                    mds_request_info* info);
int mds_server_get_stats(mds_server* s, mds_server_stats* out);
/* hold != 0: admit no queued request into a batch until called again with
 * 0 (batches already running finish; submissions keep queueing). Lets an
 * operator drain the device or gather a burst into shared batches. No
 * reference counterpart (the reference runs the Nystrom chain per file). */
int mds_server_hold(mds_server* s, int hold);

#ifdef __cplusplus
}
#endif

#endif /* MDSGPU_H */
