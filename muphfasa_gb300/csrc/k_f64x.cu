// k_f64x.cu -- the FP64-accurate step on GB300's integer pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (2 DFMA per SM per clock), so
// a D3Q19 cell update with ~170 FP64 operations is FP64-bound at ~15% of the
// HBM roofline.  This kernel keeps each population as a 64-bit fixed-point
// number h_n = f_n / w_n (resolution 2^-56 of a quantity of order one, far
// finer than FP64's 2^-53 relative rounding) and does the BGK+Guo update with
// integer adds and 64x64->high-64 multiplies (IMAD pipe):
//
//   rho = sum_k w_k S_k,  J = sum_k w_k (sum_{n in k} c_n h_n) + F/2
//   r = 1/rho (FP32 seed + one fixed-point Newton step), u = J r
//   Pi = J u  (= rho u u),  A = rho - 1.5 tr(Pi)
//   feq_n / w_n = A + 3 c_n.J + 4.5 c_n c_n : Pi              (adds only)
//   guo_n / w_n = c_n.F' + 3 (c_n.u)(c_n.F') - u.F',  F' = 3 (1 - omega/2) F
//   h_n' = h_n + omega (feq_n/w_n - h_n) + guo_n/w_n          (1 multiply)
//
// which is the reference's BGK + Guo update (Collision.cpp:55-92,
// Collision.H:21-76, Equilibrium.H:43-57) in exact arithmetic; the rounding
// of the reference's FP64 evaluation (~1e-16 per operation) is the only
// difference, so results agree to ~1e-16 per step.  The HBM traffic is the
// same 2*Q*8 bytes per cell update as FP64 storage.
//
// Range: class sums of h within +-128, rho in (1/16, 64), |J|, |u| < 4 and
// |feq/w - h| < 32; a cell outside sets the handle's error flag (reported as
// MPH_ERR_NONFINITE by the host) instead of producing silent wrap-around.
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "fx_kernels.cuh"
#include "lbm_launch.h"

namespace mph {

namespace {

// OBST: the domain has obstacles (p.cls set); the plain instantiation
// carries no class-byte test.  Launched in blocks of 128 threads along x
// (104 registers: 4 blocks, 16 warps per SM): 18.3 GLUPS at 512^3 against
// 17.9 for blocks of 256 with the same occupancy; capping the registers at
// 96 for 20 warps per SM measured 17.7.
// WIN: the launch covers the window (y0, y1, z0, z1) of p rather than the
// whole domain (the offsets cost about 1 % at 512^3 when always applied).
template <int Q, bool FORCED, bool OBST, bool WIN>
__global__ void __launch_bounds__(256) k_step_x(const i64* __restrict__ fin, i64* __restrict__ fout, const KParams p,
                                                const KParamsX px, const KParams* __restrict__ pg,
                                                const i64* __restrict__ kbb, int* __restrict__ flag) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = (WIN ? p.y0 : 0) + blockIdx.y * blockDim.y + threadIdx.y;
    const int z = (WIN ? p.z0 : 0) + blockIdx.z;
    if (x >= p.nx || y >= (WIN ? p.y1 : p.ny)) return;
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
    if (OBST && p.cls[c] == kSolid) {  // obstacle cell: rest state, h = f / w = 1
#pragma unroll
        for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = 1LL << 56;
        return;
    }
    i64 h[Q];
    pull_x<Q, OBST>(p, pg, kbb, fin, x, y, z, c, h);
    int bad = 0;
    collide_x<Q, FORCED>(px, h, bad);
    if (bad) atomicOr(flag, 1);
#pragma unroll
    for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = h[n];
}

// Persistent, software-pipelined variant.  A tile is 256 consecutive cells of
// one row (y, z); each CTA walks the tiles with a grid stride.  Before the
// collide of tile t every thread issues cp.async copies of the Q values its
// cell of tile t + gridDim.x will pull into the other shared-memory stage, so
// the HBM latency of the next tile overlaps the integer arithmetic of this
// one without extra warps.  Each thread only reads what it copied itself, so
// the per-thread cp.async.wait_group is the only synchronisation.  Cells next
// to a non-periodic face (and lanes past the row end) skip the staging and
// use the direct boundary pull.
constexpr int kPipeThreads = 256;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <int Q>
__device__ __forceinline__ void tile_cell(const KParams& p, int tiles_per_row, int tile, int& x, int& y, int& z) {
    const int row = tile / tiles_per_row;
    x = (tile - row * tiles_per_row) * kPipeThreads + threadIdx.x;
    y = row % p.ny;
    z = row / p.ny;
}

template <int Q>
__device__ __forceinline__ void stage_tile(const KParams& p, const i64* __restrict__ fin, int tiles_per_row, int tile,
                                           i64* __restrict__ buf) {
    using L = Lat<Q>;
    int x, y, z;
    tile_cell<Q>(p, tiles_per_row, tile, x, y, z);
    if (x < p.nx) {
        const Nbr o = neighbours<L::D>(p, x, y, z);
        if (!o.wall) {
            const unsigned N = (unsigned)p.ncell;
            const int ci = (z * p.ny + y) * p.nx + x;
#pragma unroll
            for (int n = 0; n < Q; ++n)
                cp_async8(buf + n * kPipeThreads + threadIdx.x, fin + ((unsigned)n * N + (unsigned)(ci + upstream<Q>(o, n))));
        }
    }
    cp_async_commit();
}

template <int Q, bool FORCED>
__global__ void __launch_bounds__(kPipeThreads) k_step_x_pipe(const i64* __restrict__ fin, i64* __restrict__ fout,
                                                              const KParams p, const KParamsX px,
                                                              const KParams* __restrict__ pg,
                                                              const i64* __restrict__ kbb, int* __restrict__ flag,
                                                              int tiles_per_row, int ntiles) {
    using L = Lat<Q>;
    extern __shared__ i64 smem[];  // [2][Q][kPipeThreads]
    int stage = 0;
    int tile = blockIdx.x;
    if (tile < ntiles) stage_tile<Q>(p, fin, tiles_per_row, tile, smem);
    int bad = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        const int next = tile + gridDim.x;
        if (next < ntiles) stage_tile<Q>(p, fin, tiles_per_row, next, smem + (stage ^ 1) * Q * kPipeThreads);
        else cp_async_commit();
        cp_async_wait1();
        int x, y, z;
        tile_cell<Q>(p, tiles_per_row, tile, x, y, z);
        if (x < p.nx) {
            const long long c = ((long long)z * p.ny + y) * p.nx + x;
            const Nbr o = neighbours<L::D>(p, x, y, z);
            i64 h[Q];
            if (!o.wall) {
                const i64* b = smem + stage * Q * kPipeThreads + threadIdx.x;
#pragma unroll
                for (int n = 0; n < Q; ++n) h[n] = b[n * kPipeThreads];
            } else {
                pull_x<Q, false>(p, pg, kbb, fin, x, y, z, c, h);
            }
            collide_x<Q, FORCED>(px, h, bad);
            const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
            for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = h[n];
        }
        stage ^= 1;
    }
    if (bad) atomicOr(flag, 1);
}

}  // namespace

namespace {
template <int Q, bool FORCED, bool OBST, bool WIN>
void step_x_launch(const i64* fin, i64* fout, const KParams& p, const KParamsX& px, const KParams* pg, const i64* kbb,
                   int* flag, cudaStream_t s) {
    dim3 g, b;
    step_shape(p, g, b, 128);
    if (const char* env = std::getenv("MPH_F64X_BLOCK")) {  // "BXxBY": other block shapes
        int bx = 0, by = 0;
        if (std::sscanf(env, "%dx%d", &bx, &by) == 2 && bx >= 32 && bx % 32 == 0 && by >= 1 && bx * by <= 256) {
            b = dim3(bx, by, 1);
            g = dim3((p.nx + bx - 1) / bx, (p.y1 - p.y0 + by - 1) / by, p.z1 - p.z0);
        }
    }
    k_step_x<Q, FORCED, OBST, WIN><<<g, b, 0, s>>>(fin, fout, p, px, pg, kbb, flag);
}

template <class F>
cudaError_t with_q(int q, F&& f) {
    switch (q) {
        case 9: return f(std::integral_constant<int, 9>{});
        case 15: return f(std::integral_constant<int, 15>{});
        case 19: return f(std::integral_constant<int, 19>{});
        case 27: return f(std::integral_constant<int, 27>{});
    }
    return cudaErrorInvalidValue;
}

// Three run-time flags to compile-time constants.
template <class F>
cudaError_t with_flags(bool a, bool b, bool c, F&& f) {
    using T = std::true_type;
    using N = std::false_type;
    if (a) {
        if (b) return c ? f(T{}, T{}, T{}) : f(T{}, T{}, N{});
        return c ? f(T{}, N{}, T{}) : f(T{}, N{}, N{});
    }
    if (b) return c ? f(N{}, T{}, T{}) : f(N{}, T{}, N{});
    return c ? f(N{}, N{}, T{}) : f(N{}, N{}, N{});
}

template <int Q, bool FORCED>
cudaError_t pipe_setup(size_t& smem) {
    smem = 2 * Q * kPipeThreads * sizeof(long long);
    return cudaFuncSetAttribute(k_step_x_pipe<Q, FORCED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace

int f64x_pipe_ctas(int q, bool forced) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    size_t smem = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define MPH_XP_OCC(QQ)                                                                                         \
    case QQ:                                                                                                   \
        e = forced ? pipe_setup<QQ, true>(smem) : pipe_setup<QQ, false>(smem);                                 \
        if (e == cudaSuccess)                                                                                  \
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                                 \
                &per_sm, forced ? k_step_x_pipe<QQ, true> : k_step_x_pipe<QQ, false>, kPipeThreads, smem);    \
        break;
    switch (q) {
        MPH_XP_OCC(9)
        MPH_XP_OCC(15)
        MPH_XP_OCC(19)
        MPH_XP_OCC(27)
    }
#undef MPH_XP_OCC
    if (e != cudaSuccess) return 0;
    return per_sm * sms;
}

cudaError_t launch_step_f64x_pipe(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                                  const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                                  int ctas, cudaStream_t s) {
    const int tiles_per_row = (p.nx + kPipeThreads - 1) / kPipeThreads;
    const int ntiles = tiles_per_row * p.ny * p.nz;
    const int grid = ctas < ntiles ? ctas : ntiles;
    const size_t sm = 2 * (size_t)q * kPipeThreads * sizeof(long long);
#define MPH_XP_CASE(QQ)                                                                                       \
    case QQ:                                                                                                  \
        if (forced)                                                                                           \
            k_step_x_pipe<QQ, true><<<grid, kPipeThreads, sm, s>>>(fin, fout, p, px, pg, kbb, flag, tiles_per_row, ntiles);  \
        else                                                                                                  \
            k_step_x_pipe<QQ, false><<<grid, kPipeThreads, sm, s>>>(fin, fout, p, px, pg, kbb, flag, tiles_per_row, ntiles); \
        return cudaGetLastError();
    switch (q) {
        MPH_XP_CASE(9)
        MPH_XP_CASE(15)
        MPH_XP_CASE(19)
        MPH_XP_CASE(27)
    }
#undef MPH_XP_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_step_f64x(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                             const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                             cudaStream_t s) {
    const bool win = p.y0 != 0 || p.y1 != p.ny || p.z0 != 0 || p.z1 != p.nz;
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        return with_flags(forced, p.cls != nullptr, win, [&](auto fc, auto oc, auto wc) {
            step_x_launch<Q, decltype(fc)::value, decltype(oc)::value, decltype(wc)::value>(fin, fout, p, px, pg,
                                                                                            kbb, flag, s);
            return cudaGetLastError();
        });
    });
}

}  // namespace mph
