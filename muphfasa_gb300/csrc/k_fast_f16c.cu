// k_fast_f16c.cu -- shifted custom 16-bit float storage (f - w in the 1-4-11
// format of StF16C), FP32 arithmetic (single domain and batch).
#include "batch_kernel.cuh"
#include "bulk_step.cuh"
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f16c(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF16C>(q, forced, fin, fout, p, pg, s);
}
cudaError_t launch_step_bulk_f16c(int mode, int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, long long total_elems, int cells, int stages, int* flag,
                                  cudaStream_t s) {
    return launch_step_bulk_t<StF16C>(mode, q, forced, fin, fout, p, pg, total_elems, cells, stages, flag, s);
}
cudaError_t launch_batch_f16c(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks, int nchunks,
                       const int2* walls, int nwalls, const KParams* dp, const long long* offs, cudaStream_t s) {
    return launch_batch_t<StF16C, kFast>(q, forced, K, persistent, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
}
cudaError_t launch_batch_bulk_f16c(int mode, int q, bool forced, int stages, int lpad, const void* fin, void* fout,
                                   const RowChunk* chunks, int nchunks, const int2* walls, int nwalls,
                                   const KParams* dp, const long long* offs, int* flag, cudaStream_t s) {
    return launch_batch_bulk_t<StF16C>(mode, q, forced, stages, lpad, fin, fout, chunks, nchunks, walls, nwalls, dp, offs,
                                     flag, s);
}
}  // namespace mph
