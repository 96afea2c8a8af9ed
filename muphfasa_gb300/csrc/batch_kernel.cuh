// batch_kernel.cuh -- the step kernel over a flat list of tiles of many
// independent domains (batch.cu).  Shared between batch.cu and the FP64
// exact translation unit, which instantiates it with the reference's
// arithmetic (no FMA contraction).
#pragma once
#include <utility>

#include "lbm_kernels.cuh"

namespace mph {

struct Tile {  // one block: a width x (256 / width) patch of one z-plane of domain dom
    int dom, x0, y0, z0;
};

namespace {

template <int Q, class St, int ARITH, bool FORCED>
__global__ void __launch_bounds__(256) k_batch_step(const typename St::T* __restrict__ fin_base,
                                                    typename St::T* __restrict__ fout_base,
                                                    const Tile* __restrict__ tiles, const KParams* __restrict__ dp,
                                                    const long long* __restrict__ offs) {
    const Tile t = tiles[blockIdx.x];
    const KParams& p = dp[t.dom];
    const int x = t.x0 + threadIdx.x;
    const int y = t.y0 + threadIdx.y;
    const int z = t.z0;
    if (x >= p.nx || y >= p.ny) return;
    const long long off = offs[t.dom];
    step_cell<Q, St, ARITH, FORCED>(p, &p, fin_base + off, fout_base + off, x, y, z);
}

template <class F>
cudaError_t batch_with_q(int q, F&& f) {
    switch (q) {
        case 9: return f(std::integral_constant<int, 9>{});
        case 15: return f(std::integral_constant<int, 15>{});
        case 19: return f(std::integral_constant<int, 19>{});
        case 27: return f(std::integral_constant<int, 27>{});
    }
    return cudaErrorInvalidValue;
}

template <class St, int ARITH>
cudaError_t launch_batch_t(int q, bool forced, const void* fin, void* fout, const Tile* tiles, int ntiles, dim3 block,
                           const KParams* dp, const long long* offs, cudaStream_t s) {
    return batch_with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        auto in = static_cast<const typename St::T*>(fin);
        auto out = static_cast<typename St::T*>(fout);
        if (forced) k_batch_step<Q, St, ARITH, true><<<ntiles, block, 0, s>>>(in, out, tiles, dp, offs);
        else k_batch_step<Q, St, ARITH, false><<<ntiles, block, 0, s>>>(in, out, tiles, dp, offs);
        return cudaGetLastError();
    });
}

}  // namespace

// The FP64 exact instantiation, defined in the exact translation unit.
cudaError_t launch_batch_exact(int q, bool forced, const double* fin, double* fout, const Tile* tiles, int ntiles,
                               dim3 block, const KParams* dp, const long long* offs, cudaStream_t s);

}  // namespace mph
