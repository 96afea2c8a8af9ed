// k_fast_common.cuh -- launcher template of the refactored (FMA) step
// kernels, instantiated per storage precision by k_fast_*.cu.
#pragma once

#include <cstdlib>

#include "lbm_launch.h"

namespace mph {

template <class St>
cudaError_t launch_step_fast(int q, bool forced, const void* fin, void* fout, const KParams& p, const KParams* pg,
                             cudaStream_t s) {
    dim3 g, b;
    step_shape(p, g, b);
    auto in = static_cast<const typename St::T*>(fin);
    auto out = static_cast<typename St::T*>(fout);
    if constexpr (St::kShift) {
        // Pairs of cells are read and written as 32-bit words: nx even makes
        // every pair offset even, and both arrays must be 4-byte aligned.
        const bool aligned = ((reinterpret_cast<unsigned long long>(fin) | reinterpret_cast<unsigned long long>(fout)) & 3) == 0;
        if (p.nx % 2 == 0 && aligned) {
            KParams half = p;
            half.nx = p.nx / 2;
            // Blocks of 64 pair threads (24 warps per SM either way by registers):
            // 62.8 / 63.8 GLUPS f16s / bf16s at 512^3 against 61.3 / 62.0 with 256.
            int threads = 64;  // MPH_PAIR_THREADS: 64, 128 or 256 threads per block
            if (const char* env = std::getenv("MPH_PAIR_THREADS")) {
                const int t = std::atoi(env);
                if (t == 64 || t == 128 || t == 256) threads = t;
            }
            step_shape(half, g, b, threads);  // one thread per cell pair
#define MPH_PAIR_CASE(QQ)                                                              \
    case QQ:                                                                           \
        if (forced) k_step_pair<QQ, St, true><<<g, b, 0, s>>>(in, out, p, pg);         \
        else k_step_pair<QQ, St, false><<<g, b, 0, s>>>(in, out, p, pg);               \
        return cudaGetLastError();
            switch (q) {
                MPH_PAIR_CASE(9)
                MPH_PAIR_CASE(15)
                MPH_PAIR_CASE(19)
                MPH_PAIR_CASE(27)
            }
#undef MPH_PAIR_CASE
            return cudaErrorInvalidValue;
        }
    }
#define MPH_FAST_CASE(QQ)                                                              \
    case QQ:                                                                           \
        if (forced) k_step<QQ, St, kFast, true><<<g, b, 0, s>>>(in, out, p, pg);      \
        else k_step<QQ, St, kFast, false><<<g, b, 0, s>>>(in, out, p, pg);            \
        return cudaGetLastError();
    switch (q) {
        MPH_FAST_CASE(9)
        MPH_FAST_CASE(15)
        MPH_FAST_CASE(19)
        MPH_FAST_CASE(27)
    }
#undef MPH_FAST_CASE
    return cudaErrorInvalidValue;
}

}  // namespace mph
