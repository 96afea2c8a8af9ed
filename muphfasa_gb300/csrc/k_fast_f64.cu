// k_fast_f64.cu -- FP64 storage, refactored FMA arithmetic (single domain
// and batch).
#include "batch_kernel.cuh"
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f64(int q, bool forced, const double* fin, double* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF64>(q, forced, fin, fout, p, pg, s);
}
cudaError_t launch_batch_fast_f64(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks, int nchunks,
                       const int2* walls, int nwalls, const KParams* dp, const long long* offs, cudaStream_t s) {
    return launch_batch_t<StF64, kFast>(q, forced, K, persistent, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
}
}  // namespace mph
