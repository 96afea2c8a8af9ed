// k_fast_f16.cu -- shifted FP16 / BF16 storage (f - w), FP32 arithmetic.
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f16s(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF16S>(q, forced, fin, fout, p, pg, s);
}
cudaError_t launch_step_fast_bf16s(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                   const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StBF16S>(q, forced, fin, fout, p, pg, s);
}
}  // namespace mph
