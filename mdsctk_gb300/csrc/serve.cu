// serve.cu -- resident Nystrom serving loop on sm_103a.
//
// The reference runs out-of-sample extension as a file pipeline
// (examples/cluster_rms_nystrom.bash:54-66): knn_rms -r landmarks -f queries
// (the nearest landmark of each query is dropped, knn_rms.cpp:248-249),
// make_gesparse, decomp_sparse_nystrom (B = exp(-d^2/2s^2) scaled by the
// landmark degrees d_a and the query's own column sum d_b, ext = B^T z/lambda,
// decomp_sparse_nystrom.cpp:181-219,301-312). Here the landmark model (prepared
// frames, template, tensor-core operands, kNN graph, eigenpairs, degrees)
// stays on the device, and query requests of any size are served by:
//
//  * slots: S independent workspaces, each with its own context (stream,
//    buffer cache) sized for `max_batch_frames`; S is set by the HBM budget.
//  * continuous batching: a scheduler thread admits queued requests into a
//    free slot (FIFO, whole requests, up to the slot's capacity) while other
//    slots' batches are still on the GPU, so batches overlap on the device.
//  * CUDA graphs: the batch pipeline (centring, superposition onto the
//    landmark template, split-precision operands, candidate screen against
//    the landmarks, exact recheck, Nystrom extension, result copies) is
//    captured once per (slot, size bucket) and replayed; the batch is padded
//    to its bucket with zero frames whose results are ignored.
//  * the rare rows whose screen guard fails are finished on the host side of
//    the slot (wider screen, exact rows) before results are published.
//
// A request's results depend only on its own frames: every kernel works per
// query row, so a request gives the same output alone or batched with others.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "knn_common.cuh"
#include "qcp.cuh"

int decomp_resident(mds_ctx* ctx, int n, const int* dpcol, const int* dirow, const double* ddist, double sigma,
                    int nev, int ncv, double tol, int maxiter, std::vector<double>& evals, double* dZ, double* ddinv,
                    int* nconv);

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Nystrom extension of one batch: one thread per query. The query's column of
// the general matrix holds its k neighbours in ascending landmark order
// (make_gesparse's cursor order); sums run in that order.
__global__ void k_serve_ext(const double* __restrict__ d, const int* __restrict__ idx, int m, int k, double sigma,
                            const double* __restrict__ dinv_a, const double* __restrict__ Z, int n,
                            const double* __restrict__ lam, int nev, double* __restrict__ ext) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const double* dq = d + (int64_t)q * k;
  const int* iq = idx + (int64_t)q * k;
  // selection order: ascending landmark index (k is small; no duplicates)
  int prev = -1;
  double sb = 0.0;
  for (int t = 0; t < k; ++t) {
    int best = -1;
    for (int p = 0; p < k; ++p)
      if (iq[p] > prev && (best < 0 || iq[p] < iq[best])) best = p;
    prev = iq[best];
    double a = dq[best];
    sb += exp(-(a * a) / (2.0 * sigma * sigma));
  }
  const double db = 1.0 / sqrt(sb);
  for (int x = 0; x < nev; ++x) {
    double e = 0.0;
    prev = -1;
    for (int t = 0; t < k; ++t) {
      int best = -1;
      for (int p = 0; p < k; ++p)
        if (iq[p] > prev && (best < 0 || iq[p] < iq[best])) best = p;
      prev = iq[best];
      double a = dq[best];
      double b = exp(-(a * a) / (2.0 * sigma * sigma)) * (dinv_a[prev] * db);
      e += b * (Z[(int64_t)x * n + prev] / lam[x]);
    }
    ext[(int64_t)q * nev + x] = e;
  }
}

struct Request {
  int64_t ticket = 0;
  int m = 0;
  std::vector<float> xyz;
  std::vector<double> ext, d;
  std::vector<int> idx;
  double t_submit = 0, t_start = 0, t_done = 0;
  int batch = -1, batch_frames = 0, status = MDS_OK, rows_flagged = 0;
  bool done = false;
};

struct Slot {
  mds_ctx* ctx = nullptr;
  int cap = 0;
  DevBuf raw, A, R, cand, cand_n, out_d, out_i, flagged, nflag, derr, ext, lb, rowthr;
  DevBuf audit;  // the recheck's audit counters of the screen's bounds (4 x u64)
  TcOperands tcq;
  float* h_raw = nullptr;
  double* h_d = nullptr;
  double* h_ext = nullptr;
  int* h_i = nullptr;
  int* h_small = nullptr;  // [0] flagged rows, [1] screen error, [2] pivot-pass error
  int* h_flagrows = nullptr;
  cudaEvent_t done = nullptr;
  std::map<int, cudaGraphExec_t> graphs;
  std::map<int, bool> warmed;
  std::vector<std::shared_ptr<Request>> reqs;
  int m = 0, bucket = 0, batch = -1;
  bool busy = false;
};

const int kBuckets[] = {1, 2, 4, 8, 16, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096,
                        6144, 8192, 12288, 16384};

}  // namespace

struct mds_server {
  mds_server_config cfg{};
  mds_ctx* main = nullptr;
  std::string last_error;
  int n = 0, natoms = 0, Ap = 0, k = 0, nev = 0, Kp = 0, nseg_max = 1, segstride = 0;
  unsigned prec = MDS_PREC_FP32;
  float tm = 0;
  DevBuf dmass, dswn, dmu, dM0, Y, E, A, R, U, dZ, ddinv, dlam;
  DevBuf nmax;  // largest |a|^2 of the landmarks (tensor-core screen thresholds)
  TcPivots pv;  // landmark pivots for tile skipping (pv.nC = 0: off)
  TcOperands tc;
  std::vector<double> evals;
  std::list<Slot> slots;  // slots own device buffers and never move
  std::deque<std::shared_ptr<Request>> queue;
  std::map<int64_t, std::shared_ptr<Request>> reqs;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  bool hold = false;  // mds_server_hold: admit nothing while set
  int64_t next_ticket = 1;
  mds_server_stats st{};
  KnnRmsPlan plan(int nfit) const {
    KnnRmsPlan p;
    p.nref = n;
    p.nfit = nfit;
    p.natoms = natoms;
    p.Ap = Ap;
    p.k = k;
    p.kprime = Kp;
    p.nofit = (cfg.flags & MDS_NOFIT) ? 1 : 0;
    p.prec = prec;
    p.guard_fp32 = MDS_GUARD_FP32;
    p.guard_tc = MDS_GUARD_TC;
    return p;
  }
};

static int srv_fail(mds_server* s, int code, const char* msg) {
  s->last_error = msg;
  return code;
}

static int bucket_for(int m) {
  for (int b : kBuckets)
    if (b >= m) return b;
  return m;
}

// The batch pipeline on the slot's stream (capturable: no allocation that
// misses the cache, no synchronisation).
static int launch_batch(mds_server* S, Slot& sl, int bucket) {
  mds_ctx* c = sl.ctx;
  KnnRmsPlan pl = S->plan(bucket);
  MDS_CUDA(c, cudaMemsetAsync(sl.nflag.p, 0, sizeof(int), c->stream));
  MDS_CUDA(c, cudaMemsetAsync(sl.audit.p, 0, 4 * sizeof(unsigned long long), c->stream));
  MDS_TRY(launch_prep(c, sl.raw.as<float>(), bucket, S->natoms, S->Ap, S->dmass.as<float>(), S->dswn.as<float>(),
                      S->tm, S->dmu.as<float>(), S->dM0.as<double>(), pl.nofit, sl.A.as<float>(), sl.R.as<float>()));
  int nseg;
  if (S->prec != MDS_PREC_FP32) {
    nseg = std::min(tc_choose_nseg(c, pl, bucket), S->nseg_max);
    MDS_TRY(tc_prepare(c, pl, sl.A.as<float>(), bucket, sl.tcq, 0));
    TcSkip sk;
    if (S->pv.nC > 0) {  // tile skipping: bounds of the batch's frames to the landmark pivots
      MDS_TRY(tc_skip_bounds(c, pl, sl.tcq, sl.R.as<float>(), bucket, S->pv, sl.lb.as<float>(),
                             sl.derr.as<int>() + 2));
      sk.pivlb = sl.lb.as<float>();
      sk.prad = S->pv.rad.as<float>();
    }
    MDS_TRY(launch_screen_tc(c, pl, sl.tcq, S->tc, sl.R.as<float>(), S->R.as<float>(), bucket, S->Kp, nseg,
                             sl.cand.as<uint64_t>(), sl.cand_n.as<int>(), sl.derr.as<int>(),
                             S->pv.nC > 0 ? &sk : nullptr, nullptr, sl.rowthr.as<float>(), S->nmax.as<float>()));
  } else {
    nseg = std::min(choose_nseg_fp32(bucket, c->num_sms, S->n), S->nseg_max);
    MDS_CUDA(c, cudaMemsetAsync(sl.derr.p, 0, sizeof(int), c->stream));
    MDS_TRY(launch_screen_fp32(c, pl, sl.A.as<float>(), S->A.as<float>(), sl.R.as<float>(), S->R.as<float>(), bucket,
                               nullptr, S->Kp, nseg, sl.cand.as<uint64_t>(), sl.cand_n.as<int>()));
  }
  const int segstride = (S->prec == MDS_PREC_FP32) ? S->Kp : tc_seg_stride();
  // the recheck audits the screen's bounds on the pairs it rechecks; a row
  // with a bound above its exact value is flagged and finished like a row
  // whose guard check failed (finish_batch)
  RecheckAudit audit;
  audit.recf = sl.R.as<float>();
  audit.recr = S->R.as<float>();
  audit.guard = (S->prec == MDS_PREC_FP32) ? pl.guard_fp32 : pl.guard_tc;
  audit.counters = sl.audit.as<unsigned long long>();
  MDS_TRY(launch_recheck(c, pl, sl.A.as<float>(), S->A.as<float>(), S->dmu.as<float>(), S->U.as<float>(), bucket,
                         nullptr, 0, sl.cand.as<uint64_t>(), sl.cand_n.as<int>(), nseg, segstride, S->Kp, S->k,
                         sl.out_d.as<double>(), sl.out_i.as<int>(), sl.flagged.as<int>(), sl.nflag.as<int>(),
                         S->prec == MDS_PREC_FP32 ? nullptr : sl.rowthr.as<float>(), &audit));
  c->stats.launches++;
  k_serve_ext<<<(bucket + 127) / 128, 128, 0, c->stream>>>(sl.out_d.as<double>(), sl.out_i.as<int>(), bucket, S->k,
                                                          S->cfg.sigma, S->ddinv.as<double>(), S->dZ.as<double>(),
                                                          S->n, S->dlam.as<double>(), S->nev, sl.ext.as<double>());
  MDS_CUDA(c, cudaGetLastError());
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_d, sl.out_d.p, sizeof(double) * (size_t)bucket * S->k, cudaMemcpyDeviceToHost,
                              c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_i, sl.out_i.p, sizeof(int) * (size_t)bucket * S->k, cudaMemcpyDeviceToHost,
                              c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_ext, sl.ext.p, sizeof(double) * (size_t)bucket * S->nev,
                              cudaMemcpyDeviceToHost, c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_small, sl.nflag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_small + 1, sl.derr.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_small + 2, sl.derr.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
  return MDS_OK;
}

// Host side of a finished batch: rows whose guard failed are screened again
// (wider, many column segments), then rechecked exactly if needed; their
// extension is recomputed with the others.
static int finish_batch(mds_server* S, Slot& sl) {
  mds_ctx* c = sl.ctx;
  if (sl.h_small[1] || sl.h_small[2]) return mds_fail(c, MDS_ERR_TIMEOUT, "screen reported a timed-out wait");
  int nf = sl.h_small[0];
  if (nf <= 0) return MDS_OK;
  std::vector<int> rows(nf);
  MDS_CUDA(c, cudaMemcpyAsync(rows.data(), sl.flagged.p, sizeof(int) * nf, cudaMemcpyDeviceToHost, c->stream));
  MDS_CUDA(c, cudaStreamSynchronize(c->stream));
  std::vector<int> keep;
  for (int r : rows)
    if (r < sl.m) keep.push_back(r);  // padding rows are ignored
  if (keep.empty()) return MDS_OK;
  std::sort(keep.begin(), keep.end());
  S->st.rows_flagged += (long long)keep.size();
  const int h = (int)keep.size();
  KnnRmsPlan pl = S->plan(sl.bucket);
  DevBuf drows(c), cand(c), cand_n(c);
  MDS_TRY(drows.alloc(c, sizeof(int) * h));
  MDS_CUDA(c, cudaMemcpyAsync(drows.p, keep.data(), sizeof(int) * h, cudaMemcpyHostToDevice, c->stream));
  int Kp = std::min(S->Kp * 4, 448);
  int nflag = h;
  if (Kp < S->n) {
    const int nrt2 = (h + 31) / 32;
    const int nseg2 = std::max(1, std::min((2 * c->num_sms + nrt2 - 1) / nrt2, (S->n + 63) / 64));
    MDS_TRY(cand.alloc(c, sizeof(uint64_t) * (size_t)h * nseg2 * Kp));
    MDS_TRY(cand_n.alloc(c, sizeof(int) * (size_t)h * nseg2));
    MDS_CUDA(c, cudaMemsetAsync(sl.nflag.p, 0, sizeof(int), c->stream));
    MDS_TRY(launch_screen_fp32(c, pl, sl.A.as<float>(), S->A.as<float>(), sl.R.as<float>(), S->R.as<float>(), h,
                               drows.as<int>(), Kp, nseg2, cand.as<uint64_t>(), cand_n.as<int>()));
    MDS_TRY(launch_recheck(c, pl, sl.A.as<float>(), S->A.as<float>(), S->dmu.as<float>(), S->U.as<float>(), h,
                           drows.as<int>(), 0, cand.as<uint64_t>(), cand_n.as<int>(), nseg2, Kp, Kp, S->k,
                           sl.out_d.as<double>(), sl.out_i.as<int>(), sl.flagged.as<int>(), sl.nflag.as<int>()));
    MDS_CUDA(c, cudaMemcpyAsync(&nflag, sl.nflag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MDS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nflag > 0) {
      MDS_CUDA(c, cudaMemcpyAsync(rows.data(), sl.flagged.p, sizeof(int) * nflag, cudaMemcpyDeviceToHost, c->stream));
      MDS_CUDA(c, cudaStreamSynchronize(c->stream));
      keep.assign(rows.begin(), rows.begin() + nflag);
      MDS_CUDA(c, cudaMemcpyAsync(drows.p, keep.data(), sizeof(int) * nflag, cudaMemcpyHostToDevice, c->stream));
    }
  }
  if (nflag > 0)
    MDS_TRY(launch_recheck(c, pl, sl.A.as<float>(), S->A.as<float>(), S->dmu.as<float>(), S->U.as<float>(), nflag,
                           drows.as<int>(), 1, nullptr, nullptr, 1, 1, 1, S->k, sl.out_d.as<double>(),
                           sl.out_i.as<int>(), sl.flagged.as<int>(), sl.nflag.as<int>()));
  k_serve_ext<<<(sl.bucket + 127) / 128, 128, 0, c->stream>>>(
      sl.out_d.as<double>(), sl.out_i.as<int>(), sl.bucket, S->k, S->cfg.sigma, S->ddinv.as<double>(),
      S->dZ.as<double>(), S->n, S->dlam.as<double>(), S->nev, sl.ext.as<double>());
  MDS_CUDA(c, cudaGetLastError());
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_d, sl.out_d.p, sizeof(double) * (size_t)sl.m * S->k, cudaMemcpyDeviceToHost,
                              c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_i, sl.out_i.p, sizeof(int) * (size_t)sl.m * S->k, cudaMemcpyDeviceToHost,
                              c->stream));
  MDS_CUDA(c, cudaMemcpyAsync(sl.h_ext, sl.ext.p, sizeof(double) * (size_t)sl.m * S->nev, cudaMemcpyDeviceToHost,
                              c->stream));
  MDS_CUDA(c, cudaStreamSynchronize(c->stream));
  return MDS_OK;
}

// Start a batch on a free slot: stage the frames, run the (captured) pipeline.
static int start_batch(mds_server* S, Slot& sl) {
  mds_ctx* c = sl.ctx;
  cudaSetDevice(c->device);
  size_t fr = (size_t)S->natoms * 3;
  size_t off = 0;
  for (auto& rq : sl.reqs) {
    std::memcpy(sl.h_raw + off * fr, rq->xyz.data(), sizeof(float) * fr * rq->m);
    off += rq->m;
  }
  sl.bucket = std::min(bucket_for(sl.m), sl.cap);
  MDS_CUDA(c, cudaMemcpyAsync(sl.raw.p, sl.h_raw, sizeof(float) * fr * sl.m, cudaMemcpyHostToDevice, c->stream));
  if (sl.bucket > sl.m)
    MDS_CUDA(c, cudaMemsetAsync(sl.raw.as<float>() + fr * sl.m, 0, sizeof(float) * fr * (sl.bucket - sl.m),
                                c->stream));
  auto it = sl.graphs.find(sl.bucket);
  if (it != sl.graphs.end()) {
    MDS_CUDA(c, cudaGraphLaunch(it->second, c->stream));
    S->st.graph_launches++;
  } else {
    // first batch of this size: run it directly (warms the buffer cache and
    // kernel attributes), then capture the same sequence for later batches
    MDS_TRY(launch_batch(S, sl, sl.bucket));
    if (S->cfg.use_graphs) {
      MDS_CUDA(c, cudaStreamSynchronize(c->stream));
      cudaGraph_t g = nullptr;
      MDS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      int rc = launch_batch(S, sl, sl.bucket);
      cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (rc != MDS_OK) return rc;
      if (e != cudaSuccess) return mds_fail(c, MDS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      cudaGraphExec_t ex = nullptr;
      MDS_CUDA(c, cudaGraphInstantiate(&ex, g, 0));
      cudaGraphDestroy(g);
      sl.graphs[sl.bucket] = ex;
      S->st.graphs_captured++;
    }
  }
  MDS_CUDA(c, cudaEventRecord(sl.done, c->stream));
  return MDS_OK;
}

static void publish(mds_server* S, Slot& sl, int status) {
  double t = now_ms();
  size_t off = 0;
  std::lock_guard<std::mutex> lk(S->mu);
  for (auto& rq : sl.reqs) {
    if (status == MDS_OK) {
      rq->d.assign(sl.h_d + off * S->k, sl.h_d + (off + rq->m) * S->k);
      rq->idx.assign(sl.h_i + off * S->k, sl.h_i + (off + rq->m) * S->k);
      rq->ext.resize((size_t)rq->m * S->nev);
      // [frame][nev] on the device -> [nev][m] for the caller
      for (int q = 0; q < rq->m; ++q)
        for (int x = 0; x < S->nev; ++x) rq->ext[(size_t)x * rq->m + q] = sl.h_ext[(off + q) * S->nev + x];
    }
    rq->status = status;
    rq->t_done = t;
    rq->done = true;
    off += rq->m;
    S->st.requests_done++;
  }
  S->st.batches++;
  S->st.frames += sl.m;
  sl.reqs.clear();
  sl.busy = false;
  S->cv_done.notify_all();
}

static void worker_loop(mds_server* S) {
  cudaSetDevice(S->cfg.device);
  int batch_id = 0;
  while (true) {
    bool any_busy = false;
    for (auto& sl : S->slots) {
      if (!sl.busy) continue;
      cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) {
        any_busy = true;
        continue;
      }
      int status = (q == cudaSuccess) ? finish_batch(S, sl) : MDS_ERR_CUDA;
      if (status != MDS_OK) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->last_error = mds_last_error(sl.ctx);
      }
      publish(S, sl, status);
    }
    // admit queued requests into free slots
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && S->queue.empty() && !any_busy) break;
      for (auto& sl : S->slots) {
        if (sl.busy || S->queue.empty() || (S->hold && !S->stop)) continue;
        sl.reqs.clear();
        sl.m = 0;
        while (!S->queue.empty() && sl.m + S->queue.front()->m <= sl.cap) {
          auto rq = S->queue.front();
          S->queue.pop_front();
          rq->t_start = now_ms();
          rq->batch = batch_id;
          sl.m += rq->m;
          sl.reqs.push_back(rq);
        }
        if (sl.reqs.empty()) continue;
        for (auto& rq : sl.reqs) rq->batch_frames = sl.m;
        sl.batch = batch_id++;
        sl.busy = true;
        lk.unlock();
        int rc = start_batch(S, sl);
        lk.lock();
        if (rc != MDS_OK) {
          S->last_error = mds_last_error(sl.ctx);
          lk.unlock();
          publish(S, sl, rc);
          lk.lock();
        } else {
          any_busy = true;
        }
      }
      if (!any_busy && (S->queue.empty() || S->hold) && !S->stop) {
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    if (any_busy) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

static size_t slot_bytes(const mds_server* S, int cap) {
  size_t ap = S->Ap;
  size_t b = 0;
  b += (size_t)cap * S->natoms * 3 * 4;                     // raw
  b += (size_t)cap * 3 * ap * 4 + (size_t)cap * 64;            // A, R
  b += ((size_t)cap / 40 + 1) * 128 * 2 * ap * 2;            // split operands
  b += (size_t)cap * S->nseg_max * S->segstride * 8 + (size_t)cap * S->nseg_max * 4;
  b += (size_t)cap * S->k * 12 + (size_t)cap * S->nev * 8 + (size_t)cap * 4;
  b += (size_t)cap * S->pv.nC * 4;                            // pivot bounds
  return b + (64u << 20);
}

static int build_model(mds_server* S, const float* hxyz, const float* hmass) {
  mds_ctx* c = S->main;
  cudaStream_t s = c->stream;
  const int n = S->n, natoms = S->natoms, Ap = S->Ap;
  // masses (reset_x weights) and the sqrt(w/M) scaling
  std::vector<float> swn(Ap, 0.f);
  double M = 0;
  float tm = 0;
  for (int a = 0; a < natoms; ++a) {
    tm += hmass[a];
    M += hmass[a];
  }
  if (!(M > 0)) return mds_fail(c, MDS_ERR_ARG, "total mass must be positive");
  for (int a = 0; a < natoms; ++a) swn[a] = (float)std::sqrt((double)hmass[a] / M);
  S->tm = tm;
  MDS_TRY(S->dmass.alloc(c, sizeof(float) * natoms));
  MDS_TRY(S->dswn.alloc(c, sizeof(float) * Ap));
  MDS_CUDA(c, cudaMemcpyAsync(S->dmass.p, hmass, sizeof(float) * natoms, cudaMemcpyHostToDevice, s));
  MDS_CUDA(c, cudaMemcpyAsync(S->dswn.p, swn.data(), sizeof(float) * Ap, cudaMemcpyHostToDevice, s));
  DevBuf raw(c);
  MDS_TRY(raw.alloc(c, sizeof(float) * 3 * (size_t)natoms * n));
  MDS_CUDA(c, cudaMemcpyAsync(raw.p, hxyz, sizeof(float) * 3 * (size_t)natoms * n, cudaMemcpyHostToDevice, s));
  // the landmark graph: knn_rms all pairs, make_sysparse, decomp_sparse
  DevBuf kd(c), ki(c), pcol(c), irow(c), val(c);
  MDS_TRY(kd.alloc(c, sizeof(double) * (size_t)n * S->k));
  MDS_TRY(ki.alloc(c, sizeof(int) * (size_t)n * S->k));
  int ku = 0;
  int rc = mds_knn_rms(c, raw.as<float>(), n, nullptr, 0, natoms, S->dmass.as<float>(), S->k,
                       S->prec | (S->cfg.flags & MDS_NOFIT) | MDS_DEVICE_IO, kd.as<double>(), ki.as<int>(), &ku);
  if (rc) return rc;
  S->st.model_knn_ms = c->stats.total_ms;
  int64_t cap = (int64_t)n * S->k, nnz = 0;
  MDS_TRY(pcol.alloc(c, sizeof(int) * (n + 1)));
  MDS_TRY(irow.alloc(c, sizeof(int) * cap));
  MDS_TRY(val.alloc(c, sizeof(double) * cap));
  rc = mds_sysparse(c, kd.as<double>(), ki.as<int>(), n, S->k, S->k, MDS_DEVICE_IO, pcol.as<int>(), irow.as<int>(),
                    val.as<double>(), cap, &nnz);
  if (rc) return rc;
  MDS_TRY(S->dZ.alloc(c, sizeof(double) * (size_t)n * S->nev));
  MDS_TRY(S->ddinv.alloc(c, sizeof(double) * n));
  int nconv = 0;
  double t0 = now_ms();
  MDS_TRY(decomp_resident(c, n, pcol.as<int>(), irow.as<int>(), val.as<double>(), S->cfg.sigma, S->nev, S->cfg.ncv,
                          S->cfg.tol, S->cfg.maxiter, S->evals, S->dZ.as<double>(), S->ddinv.as<double>(), &nconv));
  S->st.model_decomp_ms = now_ms() - t0;
  S->st.model_nconv = nconv;
  MDS_TRY(S->dlam.alloc(c, sizeof(double) * S->nev));
  MDS_CUDA(c, cudaMemcpyAsync(S->dlam.p, S->evals.data(), sizeof(double) * S->nev, cudaMemcpyHostToDevice, s));
  // resident prepared landmarks for the query screen and recheck
  MDS_TRY(S->Y.alloc(c, sizeof(float) * 3 * (size_t)Ap));  // the first landmark, centred: the template
  MDS_TRY(S->E.alloc(c, sizeof(double)));
  MDS_TRY(launch_center(c, raw.as<float>(), 1, natoms, Ap, S->dmass.as<float>(), S->dswn.as<float>(), tm,
                        S->Y.as<float>(), S->E.as<double>()));
  std::vector<double> mu;
  double M0[9];
  MDS_TRY(build_template(c, S->Y.as<float>(), Ap, natoms, (S->cfg.flags & MDS_NOFIT) != 0, mu, M0));
  MDS_TRY(S->dmu.alloc(c, sizeof(float) * 3 * Ap));
  MDS_TRY(S->dM0.alloc(c, sizeof(double) * 9));
  std::vector<float> muf(mu.begin(), mu.end());
  MDS_CUDA(c, cudaMemcpyAsync(S->dmu.p, muf.data(), sizeof(float) * 3 * Ap, cudaMemcpyHostToDevice, s));
  MDS_CUDA(c, cudaMemcpyAsync(S->dM0.p, M0, sizeof(double) * 9, cudaMemcpyHostToDevice, s));
  MDS_TRY(S->A.alloc(c, sizeof(float) * 3 * (size_t)Ap * n));
  MDS_TRY(S->R.alloc(c, sizeof(float) * MDS_REC * (size_t)n));
  MDS_TRY(S->U.alloc(c, sizeof(float) * 18 * (size_t)n));
  MDS_TRY(launch_prep(c, raw.as<float>(), n, natoms, Ap, S->dmass.as<float>(), S->dswn.as<float>(), tm,
                      S->dmu.as<float>(), S->dM0.as<double>(), (S->cfg.flags & MDS_NOFIT) ? 1 : 0, S->A.as<float>(),
                      S->R.as<float>(), (S->cfg.flags & MDS_NOFIT) ? nullptr : S->U.as<float>()));
  if (S->prec != MDS_PREC_FP32) {
    MDS_TRY(tc_prepare(c, S->plan(n), S->A.as<float>(), n, S->tc, 1));
    if ((n + 79) / 80 >= 4) MDS_TRY(tc_skip_pivots(c, S->plan(n), S->A.as<float>(), S->R.as<float>(), S->pv));
    MDS_TRY(S->nmax.alloc(c, sizeof(float)));
    MDS_TRY(tc_rec_nmax(c, S->R.as<float>(), n, S->nmax.as<float>()));
  }
  MDS_CUDA(c, cudaStreamSynchronize(s));
  return MDS_OK;
}

extern "C" int mds_server_create(const mds_server_config* cfg, const float* land_xyz, int n, int natoms,
                                 const float* mass, mds_server** out) {
  if (!cfg || !land_xyz || !mass || !out) return MDS_ERR_ARG;
  *out = nullptr;
  if (n < 2 || natoms < 1 || cfg->k < 1 || cfg->nev < 1 || !(cfg->sigma > 0)) return MDS_ERR_ARG;
  auto S = std::make_unique<mds_server>();
  S->cfg = *cfg;
  if (S->cfg.max_batch_frames <= 0) S->cfg.max_batch_frames = 4096;
  S->n = n;
  S->natoms = natoms;
  S->Ap = mds_round_up(natoms, 64);
  S->k = std::min(cfg->k, n - 1);
  S->nev = cfg->nev;
  S->prec = cfg->flags & MDS_PREC_MASK;
  // as knn_rms: off-manifold queries whose neighbours crowd within the guard
  // of one another need the deep tensor-core lists for the guard check
  S->Kp = std::min(mds_round_up(tc_kprime_want(S->k, S->prec != MDS_PREC_FP32), 32),
                   S->prec == MDS_PREC_FP32 ? 448 : 352);
  if (S->Kp < S->k + 1 + 16) return MDS_ERR_UNSUPPORTED;
  S->segstride = (S->prec == MDS_PREC_FP32) ? S->Kp : tc_seg_stride();
  S->nseg_max = 8;
  int rc = mds_create(cfg->device, 0, &S->main);
  if (rc) return rc;
  rc = build_model(S.get(), land_xyz, mass);
  if (rc) {
    S->last_error = mds_last_error(S->main);
    mds_destroy(S->main);
    return rc;
  }
  // slots: by the HBM budget (free memory, or the configured budget)
  size_t freeb = 0, total = 0;
  cudaMemGetInfo(&freeb, &total);
  size_t budget = cfg->hbm_budget ? std::min(cfg->hbm_budget, freeb) : freeb / 2;
  int cap = S->cfg.max_batch_frames;
  size_t per = slot_bytes(S.get(), cap);
  int nslots = (int)std::max<size_t>(1, std::min<size_t>(budget / per, cfg->slots > 0 ? cfg->slots : 3));
  for (int i = 0; i < nslots; ++i) S->slots.emplace_back();
  for (auto& sl : S->slots) {
    if ((rc = mds_create(cfg->device, 0, &sl.ctx))) return rc;
    sl.cap = cap;
    mds_ctx* c = sl.ctx;
    const size_t fr = (size_t)natoms * 3;
    bool ok = sl.raw.alloc(c, sizeof(float) * fr * cap) == MDS_OK &&
              sl.A.alloc(c, sizeof(float) * 3 * S->Ap * cap) == MDS_OK &&
              sl.R.alloc(c, sizeof(float) * MDS_REC * cap) == MDS_OK &&
              sl.cand.alloc(c, sizeof(uint64_t) * (size_t)cap * S->nseg_max * S->segstride) == MDS_OK &&
              sl.cand_n.alloc(c, sizeof(int) * (size_t)cap * S->nseg_max) == MDS_OK &&
              sl.out_d.alloc(c, sizeof(double) * (size_t)cap * S->k) == MDS_OK &&
              sl.out_i.alloc(c, sizeof(int) * (size_t)cap * S->k) == MDS_OK &&
              sl.flagged.alloc(c, sizeof(int) * cap) == MDS_OK && sl.nflag.alloc(c, sizeof(int)) == MDS_OK &&
              sl.audit.alloc(c, 4 * sizeof(unsigned long long)) == MDS_OK &&
              sl.derr.alloc(c, 4 * sizeof(int)) == MDS_OK && sl.rowthr.alloc(c, sizeof(float) * cap) == MDS_OK &&
              (S->pv.nC == 0 || sl.lb.alloc(c, sizeof(float) * (size_t)S->pv.nC * cap) == MDS_OK) &&
              sl.ext.alloc(c, sizeof(double) * (size_t)cap * S->nev) == MDS_OK;
    if (!ok) {
      S->last_error = mds_last_error(c);
      return MDS_ERR_NOMEM;
    }
    if (cudaMallocHost(&sl.h_raw, sizeof(float) * fr * cap) != cudaSuccess ||
        cudaMallocHost(&sl.h_d, sizeof(double) * (size_t)cap * S->k) != cudaSuccess ||
        cudaMallocHost(&sl.h_i, sizeof(int) * (size_t)cap * S->k) != cudaSuccess ||
        cudaMallocHost(&sl.h_ext, sizeof(double) * (size_t)cap * S->nev) != cudaSuccess ||
        cudaMallocHost(&sl.h_small, sizeof(int) * 4) != cudaSuccess)
      return MDS_ERR_NOMEM;
    cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
  }
  S->st.slots = nslots;
  S->st.slot_bytes = (long long)per;
  mds_server* raw = S.release();
  raw->worker = std::thread(worker_loop, raw);
  *out = raw;
  return MDS_OK;
}

extern "C" int mds_server_destroy(mds_server* S) {
  if (!S) return MDS_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  for (auto& sl : S->slots) {
    for (auto& g : sl.graphs) cudaGraphExecDestroy(g.second);
    if (sl.done) cudaEventDestroy(sl.done);
    cudaFreeHost(sl.h_raw);
    cudaFreeHost(sl.h_d);
    cudaFreeHost(sl.h_i);
    cudaFreeHost(sl.h_ext);
    cudaFreeHost(sl.h_small);
    // buffers return to the slot context's cache, then the context frees them
    sl.raw.release(); sl.A.release(); sl.R.release(); sl.cand.release();
    sl.cand_n.release(); sl.out_d.release(); sl.out_i.release(); sl.flagged.release(); sl.nflag.release();
    sl.derr.release(); sl.ext.release(); sl.tcq.A.release(); sl.tcq.B.release(); sl.lb.release(); sl.rowthr.release();
    mds_destroy(sl.ctx);
  }
  S->dmass.release(); S->dswn.release(); S->dmu.release(); S->dM0.release(); S->Y.release(); S->E.release();
  S->A.release(); S->R.release(); S->U.release(); S->dZ.release(); S->ddinv.release(); S->dlam.release(); S->tc.A.release();
  S->tc.B.release(); S->nmax.release();
  S->pv.A.release(); S->pv.R.release(); S->pv.rad.release(); S->pv.tc.A.release(); S->pv.tc.B.release();
  mds_destroy(S->main);
  delete S;
  return MDS_OK;
}

extern "C" const char* mds_server_last_error(const mds_server* S) { return S ? S->last_error.c_str() : "null"; }

extern "C" int mds_server_model(mds_server* S, double* evals, double* evecs) {
  if (!S || !evals) return MDS_ERR_ARG;
  for (int x = 0; x < S->nev; ++x) evals[x] = S->evals[x];
  if (evecs) {
    if (cudaMemcpy(evecs, S->dZ.p, sizeof(double) * (size_t)S->n * S->nev, cudaMemcpyDeviceToHost) != cudaSuccess)
      return srv_fail(S, MDS_ERR_CUDA, "copy of the eigenvectors failed");
  }
  return MDS_OK;
}

extern "C" int mds_server_submit(mds_server* S, const float* query_xyz, int m, int64_t* ticket) {
  if (!S || !query_xyz || !ticket) return MDS_ERR_ARG;
  if (m < 1 || m > S->cfg.max_batch_frames)
    return srv_fail(S, MDS_ERR_ARG, "request size outside [1, max_batch_frames]");
  auto rq = std::make_shared<Request>();
  rq->m = m;
  rq->xyz.assign(query_xyz, query_xyz + (size_t)m * S->natoms * 3);
  rq->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return srv_fail(S, MDS_ERR_ARG, "server is stopping");
    rq->ticket = S->next_ticket++;
    S->queue.push_back(rq);
    S->reqs[rq->ticket] = rq;
    S->st.requests_submitted++;
  }
  S->cv_work.notify_one();
  *ticket = rq->ticket;
  return MDS_OK;
}

extern "C" int mds_server_wait(mds_server* S, int64_t ticket, int timeout_ms, double* ext, double* knn_d,
                               int32_t* knn_i, mds_request_info* info) {
  if (!S) return MDS_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return srv_fail(S, MDS_ERR_ARG, "unknown ticket");
  auto rq = it->second;
  if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(timeout_ms, 0)), [&] { return rq->done; }))
    return MDS_ERR_TIMEOUT;
  S->reqs.erase(it);
  if (rq->status != MDS_OK) return rq->status;
  if (ext) std::memcpy(ext, rq->ext.data(), sizeof(double) * rq->ext.size());
  if (knn_d) std::memcpy(knn_d, rq->d.data(), sizeof(double) * rq->d.size());
  if (knn_i) std::memcpy(knn_i, rq->idx.data(), sizeof(int) * rq->idx.size());
  if (info) {
    info->queue_ms = rq->t_start - rq->t_submit;
    info->total_ms = rq->t_done - rq->t_submit;
    info->batch = rq->batch;
    info->batch_frames = rq->batch_frames;
  }
  return MDS_OK;
}

extern "C" int mds_server_hold(mds_server* S, int hold) {
  if (!S) return MDS_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->hold = hold != 0;
  }
  S->cv_work.notify_all();
  return MDS_OK;
}

extern "C" int mds_server_get_stats(mds_server* S, mds_server_stats* out) {
  if (!S || !out) return MDS_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  return MDS_OK;
}
