// monitor.cu -- steady-state residual norm, FP64 on the GPU, for single
// domains and batches (no counterpart in the reference, which stops on
// max_step / stop_time only).
//
// The velocity of a cell is taken from its stored populations:
// u = (sum_n c_n f_n) / (sum_n f_n) in FP64.  A call compares it with the
// field saved by the previous call and returns
//   r = ||u - u_prev||_2 / ||u||_2   (sums over cells and components)
// and saves the new field; calls k steps apart give the relative change over
// k steps, and the field is steady when r stops changing.  All sums are
// deterministic: per-block partials in a fixed order, then a fixed-order
// final pass.
#include "batch_kernel.cuh"
#include "lbm_launch.h"
#include "mph.h"

namespace mph {
namespace {

template <int Q, class St>
__device__ __forceinline__ void stored_velocity(const typename St::T* __restrict__ f, long long c, long long N,
                                                double u[3]) {
    using L = Lat<Q>;
    double rho = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const double v = (double)St::template ld<Q>(f, n, c, N);
        rho += v;
        if (L::cx(n)) j[0] += L::cx(n) * v;
        if (L::cy(n)) j[1] += L::cy(n) * v;
        if (L::cz(n)) j[2] += L::cz(n) * v;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = j[d] / rho;
}

// Block sums of (diff^2, u^2) into part[2 * blockIdx.x + {0, 1}].
__device__ __forceinline__ void block_sums2(double a0, double a1, double* __restrict__ part) {
    __shared__ double sh[2][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, off);
        a1 += __shfl_down_sync(0xffffffffu, a1, off);
    }
    if (lane == 0) { sh[0][wid] = a0; sh[1][wid] = a1; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
        part[2 * blockIdx.x + threadIdx.x] = v;
    }
}

template <int Q, class St>
__global__ void __launch_bounds__(256) k_residual_partial(const typename St::T* __restrict__ f, long long N,
                                                          double* __restrict__ uprev, int first,
                                                          double* __restrict__ part) {
    using L = Lat<Q>;
    double a0 = 0.0, a1 = 0.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        double u[3];
        stored_velocity<Q, St>(f, c, N, u);
#pragma unroll
        for (int d = 0; d < L::D; ++d) {
            if (!first) {
                const double du = u[d] - uprev[d * N + c];
                a0 += du * du;
            }
            a1 += u[d] * u[d];
            uprev[d * N + c] = u[d];
        }
    }
    block_sums2(a0, a1, part);
}

// out[0] = sum diff^2, out[1] = sum u^2 over nblocks partials, fixed order.
__global__ void k_residual_final(const double* __restrict__ part, int first_block, int nblocks, double* __restrict__ out) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 2) return;
    double v = 0.0;
    for (int b = first_block + lane; b < first_block + nblocks; b += 32) v += part[2 * b + k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) out[2 * blockIdx.x + k] = v;
}

// Batch: one block per chunk of the batch's chunk list (256 K cells).
template <int Q, class St>
__global__ void __launch_bounds__(256) k_batch_residual_partial(const typename St::T* __restrict__ f_base,
                                                                const Chunk* __restrict__ chunks, int K,
                                                                const KParams* __restrict__ dp,
                                                                const long long* __restrict__ offs,
                                                                const long long* __restrict__ coffs,
                                                                double* __restrict__ uprev_base, int first,
                                                                double* __restrict__ part) {
    using L = Lat<Q>;
    const Chunk ch = chunks[blockIdx.x];
    const long long N = dp[ch.dom].ncell;
    const typename St::T* f = f_base + offs[ch.dom];
    double* uprev = uprev_base + L::D * coffs[ch.dom];
    double a0 = 0.0, a1 = 0.0;
    for (int k = 0; k < K; ++k) {
        const long long c = (long long)ch.c0 + threadIdx.x + 256 * k;
        if (c >= N) break;
        double u[3];
        stored_velocity<Q, St>(f, c, N, u);
#pragma unroll
        for (int d = 0; d < L::D; ++d) {
            if (!first) {
                const double du = u[d] - uprev[d * N + c];
                a0 += du * du;
            }
            a1 += u[d] * u[d];
            uprev[d * N + c] = u[d];
        }
    }
    block_sums2(a0, a1, part);
}

__global__ void k_batch_residual_final(const double* __restrict__ part, const int* __restrict__ chunk_first,
                                       double* __restrict__ out) {
    const int d = blockIdx.x, k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 2) return;
    const int b0 = chunk_first[d], b1 = chunk_first[d + 1];
    double v = 0.0;
    for (int b = b0 + lane; b < b1; b += 32) v += part[2 * b + k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) out[2 * d + k] = v;
}

template <class F>
cudaError_t mon_with_store(int prec, F&& f) {
    switch (prec) {
        case MPH_PREC_F64:
        case MPH_PREC_F64_FAST: return f(StF64{});
        case MPH_PREC_F32: return f(StF32{});
        case MPH_PREC_F16S: return f(StF16S{});
        case MPH_PREC_BF16S: return f(StBF16S{});
        case MPH_PREC_F16C: return f(StF16C{});
        case MPH_PREC_F16W: return f(StF16W{});
        case MPH_PREC_F64X: return f(StF64X{});
    }
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_residual(int prec, int q, const void* f, long long ncell, double* uprev, bool first, double* part,
                            int nblocks, double* out2, cudaStream_t s) {
    cudaError_t e = mon_with_store(prec, [&](auto st) {
        using St = decltype(st);
        return batch_with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_residual_partial<Q, St><<<nblocks, 256, 0, s>>>(static_cast<const typename St::T*>(f), ncell, uprev,
                                                              first ? 1 : 0, part);
            return cudaGetLastError();
        });
    });
    if (e != cudaSuccess) return e;
    k_residual_final<<<1, 64, 0, s>>>(part, 0, nblocks, out2);
    return cudaGetLastError();
}

cudaError_t launch_batch_residual(int prec, int q, const void* f_base, const Chunk* chunks, int nchunks, int K,
                                  const KParams* dp, const long long* offs, const long long* coffs, double* uprev,
                                  bool first, double* part, const int* chunk_first, int ndom, double* out,
                                  cudaStream_t s) {
    cudaError_t e = mon_with_store(prec, [&](auto st) {
        using St = decltype(st);
        return batch_with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_batch_residual_partial<Q, St><<<nchunks, 256, 0, s>>>(static_cast<const typename St::T*>(f_base),
                                                                    chunks, K, dp, offs, coffs, uprev,
                                                                    first ? 1 : 0, part);
            return cudaGetLastError();
        });
    });
    if (e != cudaSuccess) return e;
    k_batch_residual_final<<<ndom, 64, 0, s>>>(part, chunk_first, out);
    return cudaGetLastError();
}

}  // namespace mph
