// knn_rms_tc.cu -- tcgen05 split-precision candidate screen (in progress).
#include "knn_common.cuh"

int tc_prepare(mds_ctx* ctx, const KnnRmsPlan&, const float*, int, TcOperands&) {
  return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "tensor-core screen not built yet");
}
int tc_choose_nseg(mds_ctx*, const KnnRmsPlan&, int) { return 1; }
int launch_screen_tc(mds_ctx* ctx, const KnnRmsPlan&, const TcOperands&, const TcOperands&,
                     const float*, const float*, int, int, int, uint64_t*, int*) {
  return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "tensor-core screen not built yet");
}
