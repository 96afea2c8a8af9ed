// batch_kernel.cuh -- the step kernel over many independent domains
// (batch.cu).  Shared between batch.cu and the FP64 exact translation unit,
// which instantiates it with the reference's arithmetic (no FMA contraction).
//
// Work unit: a chunk of 256 x K consecutive cells (linear index x + nx (y +
// ny z)) of one domain, so every lane has a cell whatever the domain's
// shape; only each domain's last chunk is partial.  A thread owns K cells
// 256 apart (coalesced per k) and issues the pulls of all K before the first
// collide, K x Q independent loads in flight.  The 16-bit shifted policies
// take the K cells as K/2 adjacent pairs and collide them with packed FP32x2
// arithmetic.  The chunk kernel pulls every cell through the wrapped
// neighbour offsets (no divergent boundary branch: in 2-D cavities every row
// starts and ends at a wall); a second kernel then recomputes the cells next
// to non-periodic faces from a list with the full boundary rules, writing
// over the chunk kernel's values for them.  Each cell runs the same pull /
// collide device code as a single-domain handle, so the results are
// bit-identical to it.
#pragma once
#include <utility>

#include "lbm_kernels.cuh"

namespace mph {

struct Chunk {
    int dom;  // domain index
    int c0;   // first cell (linear index within the domain)
    int x0;   // c0's coordinates: x0, and y0 | z0 << 16
    int yz;
};

// A chunk of whole rows of one domain, rows [yb, yb + r) of plane z (the
// bulk-copy staged kernel of the 16-bit storages, bulk_step.cuh).
struct RowChunk {
    int dom, z, yb, r;
};

namespace {

// Coordinates of cell c0 + l of the chunk's domain.  v / n by a float
// reciprocal is exact after one correction for v < 2^24.
__device__ __forceinline__ void chunk_cell(const KParams& p, const Chunk& ch, int l, int& x, int& y, int& z) {
    const int v = ch.x0 + l;
    int q = __float2int_rz(__int2float_rn(v) * p.inv_nx_f);
    int r = v - q * p.nx;
    if (r < 0) { r += p.nx; --q; } else if (r >= p.nx) { r -= p.nx; ++q; }
    x = r;
    const int w = (ch.yz & 0xffff) + q;
    int q2 = __float2int_rz(__int2float_rn(w) * p.inv_ny_f);
    int r2 = w - q2 * p.ny;
    if (r2 < 0) { r2 += p.ny; --q2; } else if (r2 >= p.ny) { r2 -= p.ny; ++q2; }
    y = r2;
    z = (ch.yz >> 16) + q2;
}

template <int Q, class St, int ARITH, bool FORCED, int K>
__global__ void __launch_bounds__(256) k_batch_step(const typename St::T* __restrict__ fin_base,
                                                    typename St::T* __restrict__ fout_base,
                                                    const Chunk* __restrict__ chunks, int nchunks,
                                                    const KParams* __restrict__ dp,
                                                    const long long* __restrict__ offs) {
    using R = typename St::R;
    // One chunk per block, or a persistent grid walking the list.
    for (int ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
    const Chunk ch = chunks[ci];
    const KParams& p = dp[ch.dom];
    const long long off = offs[ch.dom];
    const typename St::T* fin = fin_base + off;
    typename St::T* fout = fout_base + off;
    const unsigned N = (unsigned)p.ncell;
    if constexpr (St::kShift) {
        static_assert(K % 2 == 0, "shifted policies take cells in pairs");
        constexpr int P = K / 2;
        float2 g[P][Q];
        int ca[P];
        bool oka[P], okb[P];
        if ((p.nx & 1) == 0) {
            // nx even: a pair (c, c + 1), c even, shares its row, and N and
            // every row offset are even, so the c_x = 0 populations of both
            // cells are one aligned 32-bit word and every store is a word.
            using L = Lat<Q>;
#pragma unroll
            for (int j = 0; j < P; ++j) {
                const int l = 2 * (threadIdx.x + 256 * j);
                ca[j] = ch.c0 + l;
                oka[j] = ca[j] < (int)N;
                if (oka[j]) {
                    int x, y, z;
                    chunk_cell(p, ch, l, x, y, z);
                    const Nbr oa = neighbours<L::D>(p, x, y, z);
                    // cell x + 1 pulls through a's offsets except for the x
                    // wrap (as in k_step_pair)
                    const int dxm = x == 0 ? -p.nx : 0, dxp = x + 2 == p.nx ? -p.nx : 0;
#pragma unroll
                    for (int n = 0; n < Q; ++n) {
                        const unsigned ea = (unsigned)n * N + (unsigned)(ca[j] + upstream<Q>(oa, n));
                        if (L::cx(n) == 0) {
                            g[j][n] = sh_ld2<Q, St>(n, fin, ea);
                        } else {
                            const unsigned eb = ea + 1u + (unsigned)(L::cx(n) == 1 ? dxm : dxp);
                            g[j][n] = make_float2(sh_ld1<Q, St>(n, fin, ea), sh_ld1<Q, St>(n, fin, eb));
                        }
                    }
                }
            }
            unsigned sat = 0;
#pragma unroll
            for (int j = 0; j < P; ++j) {
                if (!oka[j]) continue;
                collide_shift<Q, A2, FORCED>(p, g[j]);
#pragma unroll
                for (int n = 0; n < Q; ++n) sh_st2<Q, St>(n, fout, (unsigned)n * N + (unsigned)ca[j], g[j][n], sat);
            }
            sh_report<St>(p, sat);
            continue;
        }
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const int l = 2 * (threadIdx.x + 256 * j);
            ca[j] = ch.c0 + l;
            oka[j] = ca[j] < (int)N;
            okb[j] = ca[j] + 1 < (int)N;
            if (oka[j]) {
                float a[Q], b[Q];
                int x, y, z;
                chunk_cell(p, ch, l, x, y, z);
                pull_shift_interior<Q, St>(p, fin, x, y, z, ca[j], a);
                if (okb[j]) {
                    chunk_cell(p, ch, l + 1, x, y, z);
                    pull_shift_interior<Q, St>(p, fin, x, y, z, ca[j] + 1, b);
                }
#pragma unroll
                for (int n = 0; n < Q; ++n) g[j][n] = make_float2(a[n], okb[j] ? b[n] : a[n]);
            }
        }
        unsigned sat = 0;
#pragma unroll
        for (int j = 0; j < P; ++j) {
            if (!oka[j]) continue;
            collide_shift<Q, A2, FORCED>(p, g[j]);
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                const unsigned e = (unsigned)n * N + (unsigned)ca[j];
                if (okb[j] && (e & 1u) == 0) {
                    sh_st2<Q, St>(n, fout, e, g[j][n], sat);
                } else {
                    sh_st1<Q, St>(n, fout, e, g[j][n].x, sat);
                    if (okb[j]) sh_st1<Q, St>(n, fout, e + 1, g[j][n].y, sat);
                }
            }
        }
        sh_report<St>(p, sat);
    } else {
        R f[K][Q];
        int cc[K];
        bool ok[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int l = threadIdx.x + 256 * k;
            cc[k] = ch.c0 + l;
            ok[k] = cc[k] < (int)N;
            if (ok[k]) {
                int x, y, z;
                chunk_cell(p, ch, l, x, y, z);
                pull_interior<Q, St>(p, fin, x, y, z, cc[k], f[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!ok[k]) continue;
            if constexpr (ARITH == kExact) collide_exact<Q, FORCED>(p, f[k]);
            else collide_fast<Q, R, FORCED>(p, f[k]);
#pragma unroll
            for (int n = 0; n < Q; ++n) St::template ste<Q>(fout, n, (unsigned)n * N + (unsigned)cc[k], f[k][n]);
        }
    }
    }
}

// Cells next to a non-periodic face: {domain, linear cell index}, one per
// thread, with the boundary rules (runs after k_batch_step on the same
// stream and overwrites those cells).
template <int Q, class St, int ARITH, bool FORCED>
__global__ void __launch_bounds__(256) k_batch_walls(const typename St::T* __restrict__ fin_base,
                                                     typename St::T* __restrict__ fout_base,
                                                     const int2* __restrict__ cells, int ncells,
                                                     const KParams* __restrict__ dp,
                                                     const long long* __restrict__ offs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const int2 w = cells[i];
    const KParams& p = dp[w.x];
    const long long off = offs[w.x];
    const int c = w.y, row = c / p.nx;
    step_cell<Q, St, ARITH, FORCED>(p, &p, fin_base + off, fout_base + off, c - row * p.nx, row % p.ny, row / p.ny);
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

// Grid of a persistent launch: resident blocks of kernel k times the SMs.
template <class Kern>
int persistent_grid(Kern k) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0) != cudaSuccess) return 0;
    return per_sm * sms;
}

// Cells per thread offered to the autotuner: K in {1, 2, 4} (pairs only for
// the shifted policies), one chunk per block or a persistent grid.  Launches
// the chunk kernel, then the wall cells.
template <class St, int ARITH>
cudaError_t launch_batch_t(int q, bool forced, int K, bool persistent, const void* fin, void* fout,
                           const Chunk* chunks, int nchunks, const int2* walls, int nwalls, const KParams* dp,
                           const long long* offs, cudaStream_t s) {
    return batch_with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        auto in = static_cast<const typename St::T*>(fin);
        auto out = static_cast<typename St::T*>(fout);
#define MPH_BK(KK)                                                                                             \
    {                                                                                                          \
        auto kern = forced ? k_batch_step<Q, St, ARITH, true, KK> : k_batch_step<Q, St, ARITH, false, KK>;     \
        int grid = nchunks;                                                                                    \
        if (persistent) {                                                                                      \
            const int g = persistent_grid(kern);                                                               \
            if (g <= 0) return cudaErrorInvalidConfiguration;                                                  \
            grid = g < nchunks ? g : nchunks;                                                                  \
        }                                                                                                      \
        kern<<<grid, 256, 0, s>>>(in, out, chunks, nchunks, dp, offs);                                         \
    }
        if (K == 4) { MPH_BK(4) }
        else if (K == 2) { MPH_BK(2) }
        else {
            if constexpr (St::kShift) return cudaErrorInvalidValue;
            else { MPH_BK(1) }
        }
#undef MPH_BK
        if (nwalls > 0) {
            const int nb = (nwalls + 255) / 256;
            if (forced) k_batch_walls<Q, St, ARITH, true><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, offs);
            else k_batch_walls<Q, St, ARITH, false><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, offs);
        }
        return cudaGetLastError();
    });
}

}  // namespace

// Instantiations, one per storage precision, each defined in the kernel
// translation unit of that precision (k_f64_exact.cu, k_fast_*.cu) so the
// builds run in parallel.
#define MPH_DECL_BATCH(NAME)                                                                                  \
    cudaError_t NAME(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks, \
                     int nchunks, const int2* walls, int nwalls, const KParams* dp, const long long* offs,        \
                     cudaStream_t s);
MPH_DECL_BATCH(launch_batch_exact)
MPH_DECL_BATCH(launch_batch_fast_f64)
MPH_DECL_BATCH(launch_batch_f32)
MPH_DECL_BATCH(launch_batch_f16s)
MPH_DECL_BATCH(launch_batch_bf16s)
MPH_DECL_BATCH(launch_batch_f16c)
MPH_DECL_BATCH(launch_batch_f16w)
#undef MPH_DECL_BATCH
// The 16-bit storages' batch step with bulk-copy staging of the pull
// operands (bulk_step.cuh): `stages` 2 or 3, lpad = elements of one staged
// run slot; mode 0 prepares the kernel (once, before any launch or capture),
// mode 1 launches the chunk kernel and the wall cells.  cudaErrorNotSupported
// when the shared memory of one block would exceed its limit.
#define MPH_DECL_BATCH_BULK(NAME)                                                                              \
    cudaError_t NAME(int mode, int q, bool forced, int stages, int lpad, const void* fin, void* fout,         \
                     const RowChunk* chunks, int nchunks, const int2* walls, int nwalls, const KParams* dp,     \
                     const long long* offs, int* flag, cudaStream_t s);
MPH_DECL_BATCH_BULK(launch_batch_bulk_f16s)
MPH_DECL_BATCH_BULK(launch_batch_bulk_bf16s)
MPH_DECL_BATCH_BULK(launch_batch_bulk_f16c)
#undef MPH_DECL_BATCH_BULK
// The fixed-point step (k_f64x_batch.cu): per-domain fixed-point constants
// dpx, bounce-back tables kbb (27 x 27 per domain) and the range flag.
cudaError_t launch_batch_f64x(int q, bool forced, int K, bool persistent, const void* fin, void* fout,
                              const Chunk* chunks, int nchunks, const int2* walls, int nwalls, const KParams* dp,
                              const KParamsX* dpx, const long long* offs, const long long* kbb, int* flag,
                              cudaStream_t s);

// Per-domain residual sums of a batch (monitor.cu): out[2 d + {0, 1}].
cudaError_t launch_batch_residual(int prec, int q, const void* f_base, const Chunk* chunks, int nchunks, int K,
                                  const KParams* dp, const long long* offs, const long long* coffs, double* uprev,
                                  bool first, double* part, const int* chunk_first, int ndom, double* out,
                                  cudaStream_t s);

}  // namespace mph
