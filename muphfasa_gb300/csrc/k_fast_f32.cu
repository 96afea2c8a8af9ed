// k_fast_f32.cu -- FP32 storage and arithmetic (single domain and batch).
#include "batch_kernel.cuh"
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f32(int q, bool forced, const float* fin, float* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF32>(q, forced, fin, fout, p, pg, s);
}
cudaError_t launch_batch_f32(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks, int nchunks,
                       const int2* walls, int nwalls, const KParams* dp, const long long* offs, cudaStream_t s) {
    return launch_batch_t<StF32, kFast>(q, forced, K, persistent, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
}
}  // namespace mph
