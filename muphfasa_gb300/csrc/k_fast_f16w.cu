// k_fast_f16w.cu -- shifted, weight-scaled custom 16-bit float storage
// ((f - w) / p in the 1-3-12 format of StF16W), FP32 arithmetic (single
// domain and batch; the bulk-copy staged kernels do not take it).
#include "batch_kernel.cuh"
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f16w(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF16W>(q, forced, fin, fout, p, pg, s);
}
cudaError_t launch_batch_f16w(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks,
                              int nchunks, const int2* walls, int nwalls, const KParams* dp, const long long* offs,
                              cudaStream_t s) {
    return launch_batch_t<StF16W, kFast>(q, forced, K, persistent, fin, fout, chunks, nchunks, walls, nwalls, dp, offs,
                                         s);
}
}  // namespace mph
