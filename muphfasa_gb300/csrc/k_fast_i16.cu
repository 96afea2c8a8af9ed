// k_fast_i16.cu -- 16-bit fixed-point storage of (f - w) / w, FP32 arithmetic
// (single domains).
#include "k_fast_common.cuh"

namespace mph {
cudaError_t launch_step_fast_i16s(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s) {
    return launch_step_fast<StI16S>(q, forced, fin, fout, p, pg, s);
}

// Range flag of the stores made by the step kernels of this translation unit.
int i16_range_flag_step(bool reset) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_range16, sizeof(int)) != cudaSuccess) return -1;
    if (reset && v) {
        const int z = 0;
        if (cudaMemcpyToSymbol(g_range16, &z, sizeof(int)) != cudaSuccess) return -1;
    }
    return v;
}
}  // namespace mph
