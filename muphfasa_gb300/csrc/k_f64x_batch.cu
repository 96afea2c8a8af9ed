// k_f64x_batch.cu -- the FP64-accurate fixed-point step (MPH_PREC_F64X) over
// a batch of independent domains (batch.cu).
//
// Same work decomposition as the other precisions' batch kernels
// (batch_kernel.cuh): a flat list of chunks of 256 K consecutive cells of one
// domain; a thread owns K cells 256 apart and issues all K x Q pulls before
// the first collide.  Every cell is pulled through the wrapped neighbour
// offsets; a second kernel recomputes the cells next to non-periodic faces
// and obstacles from a list with the full boundary rules (pull_x), writing
// over the chunk kernel's values.  The collide is collide_x of the
// single-domain kernel with the domain's own fixed-point constants, so every
// domain's result is bit-identical to a single f64x handle.  A cell leaving
// the representable range sets flag[domain]: the domains are independent,
// so the host can drop the flagged ones and keep stepping the rest.
#include "batch_kernel.cuh"
#include "fx_kernels.cuh"

namespace mph {

namespace {

template <int Q, bool FORCED, int K>
__global__ void __launch_bounds__(256) k_batch_step_x(const i64* __restrict__ fin_base, i64* __restrict__ fout_base,
                                                      const Chunk* __restrict__ chunks, int nchunks,
                                                      const KParams* __restrict__ dp,
                                                      const KParamsX* __restrict__ dpx,
                                                      const long long* __restrict__ offs, int* __restrict__ flag) {
    using L = Lat<Q>;
    // One chunk per block, or a persistent grid walking the list.
    for (int ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
        int bad = 0;
        const Chunk ch = chunks[ci];
        const KParams& p = dp[ch.dom];
        const long long off = offs[ch.dom];
        const i64* fin = fin_base + off;
        i64* fout = fout_base + off;
        const unsigned N = (unsigned)p.ncell;
        i64 h[K][Q];
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
                const Nbr o = neighbours<L::D>(p, x, y, z);
#pragma unroll
                for (int n = 0; n < Q; ++n)
                    h[k][n] = __ldg(fin + ((unsigned)n * N + (unsigned)(cc[k] + upstream<Q>(o, n))));
            }
        }
        const KParamsX px = dpx[ch.dom];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (!ok[k]) continue;
            collide_x<Q, FORCED>(px, h[k], bad);
#pragma unroll
            for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + (unsigned)cc[k]] = h[k][n];
        }
        if (bad) atomicOr(flag + ch.dom, 1);
    }
}

// Cells next to a non-periodic face or an obstacle: {domain, linear cell},
// one per thread, with the full boundary rules.  kbb holds each domain's
// 27 x 27 bounce-back constants.
template <int Q, bool FORCED>
__global__ void __launch_bounds__(256) k_batch_walls_x(const i64* __restrict__ fin_base, i64* __restrict__ fout_base,
                                                       const int2* __restrict__ cells, int ncells,
                                                       const KParams* __restrict__ dp,
                                                       const KParamsX* __restrict__ dpx,
                                                       const long long* __restrict__ offs,
                                                       const i64* __restrict__ kbb, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const int2 w = cells[i];
    const KParams& p = dp[w.x];
    const long long off = offs[w.x];
    const i64* fin = fin_base + off;
    i64* fout = fout_base + off;
    const int c = w.y, row = c / p.nx;
    const int x = c - row * p.nx, y = row % p.ny, z = row / p.ny;
    const unsigned N = (unsigned)p.ncell;
    if (p.cls && p.cls[c] == kSolid) {  // obstacle cell: rest state, h = f / w = 1
#pragma unroll
        for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + (unsigned)c] = 1LL << 56;
        return;
    }
    const i64* kb = kbb + (long long)w.x * 27 * 27;
    i64 h[Q];
    if (p.cls) pull_x<Q, true>(p, &p, kb, fin, x, y, z, c, h);
    else pull_x<Q, false>(p, &p, kb, fin, x, y, z, c, h);
    int bad = 0;
    collide_x<Q, FORCED>(dpx[w.x], h, bad);
    if (bad) atomicOr(flag + w.x, 1);
#pragma unroll
    for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + (unsigned)c] = h[n];
}

}  // namespace

// K in {1, 2} (two cells of 19-27 int64 populations each already fill the
// register file), one chunk per block or a persistent grid.  Launches the
// chunk kernel, then the wall cells.
cudaError_t launch_batch_f64x(int q, bool forced, int K, bool persistent, const void* fin, void* fout,
                              const Chunk* chunks, int nchunks, const int2* walls, int nwalls, const KParams* dp,
                              const KParamsX* dpx, const long long* offs, const long long* kbb, int* flag,
                              cudaStream_t s) {
    return batch_with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        auto in = static_cast<const i64*>(fin);
        auto out = static_cast<i64*>(fout);
#define MPH_BKX(KK)                                                                                        \
    {                                                                                                      \
        auto kern = forced ? k_batch_step_x<Q, true, KK> : k_batch_step_x<Q, false, KK>;                   \
        int grid = nchunks;                                                                                \
        if (persistent) {                                                                                  \
            const int g = persistent_grid(kern);                                                           \
            if (g <= 0) return cudaErrorInvalidConfiguration;                                              \
            grid = g < nchunks ? g : nchunks;                                                              \
        }                                                                                                  \
        kern<<<grid, 256, 0, s>>>(in, out, chunks, nchunks, dp, dpx, offs, flag);                          \
    }
        if (K == 1) { MPH_BKX(1) }
        else if (K == 2) { MPH_BKX(2) }
        else return cudaErrorInvalidValue;
#undef MPH_BKX
        if (nwalls > 0) {
            const int nb = (nwalls + 255) / 256;
            if (forced) k_batch_walls_x<Q, true><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, dpx, offs, kbb, flag);
            else k_batch_walls_x<Q, false><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, dpx, offs, kbb, flag);
        }
        return cudaGetLastError();
    });
}

}  // namespace mph
