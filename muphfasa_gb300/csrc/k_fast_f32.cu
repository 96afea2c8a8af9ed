// k_fast_f32.cu -- FP32 storage and arithmetic.
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f32(int q, bool forced, const float* fin, float* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF32>(q, forced, fin, fout, p, pg, s);
}
}  // namespace mph
