// k_fast_f16w.cu -- shifted, weight-scaled custom 16-bit float storage
// ((f - w) / w in the 1-3-12 format of StF16W), FP32 arithmetic (single
// domain; a batch does not take this storage).
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f16w(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF16W>(q, forced, fin, fout, p, pg, s);
}
}  // namespace mph
