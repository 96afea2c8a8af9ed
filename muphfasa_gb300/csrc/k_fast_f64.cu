// k_fast_f64.cu -- FP64 storage, refactored FMA arithmetic.
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_f64(int q, bool forced, const double* fin, double* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StF64>(q, forced, fin, fout, p, pg, s);
}
}  // namespace mph
