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
                            g[j][n] = St::ldr2(fin, ea);
                        } else {
                            const unsigned eb = ea + 1u + (unsigned)(L::cx(n) == 1 ? dxm : dxp);
                            g[j][n] = make_float2(St::ldr1(fin, ea), St::ldr1(fin, eb));
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < P; ++j) {
                if (!oka[j]) continue;
                collide_shift<Q, A2, FORCED>(p, g[j]);
#pragma unroll
                for (int n = 0; n < Q; ++n) St::str2(fout, (unsigned)n * N + (unsigned)ca[j], g[j][n]);
            }
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
#pragma unroll
        for (int j = 0; j < P; ++j) {
            if (!oka[j]) continue;
            collide_shift<Q, A2, FORCED>(p, g[j]);
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                const unsigned e = (unsigned)n * N + (unsigned)ca[j];
                if (okb[j] && (e & 1u) == 0) {
                    St::str2(fout, e, g[j][n]);
                } else {
                    St::str1(fout, e, g[j][n].x);
                    if (okb[j]) St::str1(fout, e + 1, g[j][n].y);
                }
            }
        }
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

// Prefetching persistent kernel for the shifted 16-bit policies (chunks of
// 512 cells, the K = 2 list): a thread owns the cell pair (2t, 2t + 1) of each
// chunk it visits and keeps a two-deep pipeline, so the HBM latency of a
// chunk's loads overlaps the collide of the previous one without more cells
// per thread:
//   iteration i: issue the 16-bit loads of chunk i + 1 (its geometry was read
//   one iteration earlier), read the geometry of chunk i + 2, collide and store
//   chunk i from the values loaded during iteration i - 1.
// Values are loaded as raw 16-bit words (the two cells of a pair may lie in
// different rows when nx is odd) and decoded with the policy's own
// conversion, so every cell gets the bits of k_batch_step.
struct ChunkGeom {
    int c0, x0, yz, nx, ny, nz, per;  // per: periodic flags, bit a for axis a
    unsigned N;
    float inx, iny;
    long long off;
};

__device__ __forceinline__ ChunkGeom chunk_geom(const Chunk* __restrict__ chunks, const KParams* __restrict__ dp,
                                                const long long* __restrict__ offs, int ci) {
    const Chunk ch = chunks[ci];
    const KParams& p = dp[ch.dom];
    ChunkGeom g;
    g.c0 = ch.c0;
    g.x0 = ch.x0;
    g.yz = ch.yz;
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.nz;
    g.per = (p.periodic[0] ? 1 : 0) | (p.periodic[1] ? 2 : 0) | (p.periodic[2] ? 4 : 0);
    g.N = (unsigned)p.ncell;
    g.inx = p.inv_nx_f;
    g.iny = p.inv_ny_f;
    g.off = offs[ch.dom];
    return g;
}

// Raw 16-bit values of the cell pair of this thread in the chunk of `g`:
// v[n] = value of cell 2t (low half) | value of cell 2t + 1 (high half).
template <int Q, class St>
__device__ __forceinline__ void pair_load(const typename St::T* __restrict__ fin_base, const ChunkGeom& g,
                                          unsigned* v) {
    using L = Lat<Q>;
    KParams q;  // the fields chunk_cell and neighbours read
    q.nx = g.nx;
    q.ny = g.ny;
    q.nz = g.nz;
    q.periodic[0] = g.per & 1;
    q.periodic[1] = (g.per >> 1) & 1;
    q.periodic[2] = (g.per >> 2) & 1;
    q.inv_nx_f = g.inx;
    q.inv_ny_f = g.iny;
    const Chunk ch{0, g.c0, g.x0, g.yz};
    const unsigned short* fin = reinterpret_cast<const unsigned short*>(fin_base + g.off);
    const int l = 2 * threadIdx.x;
    const int ca = g.c0 + l;
    const bool oka = ca < (int)g.N, okb = ca + 1 < (int)g.N;
    int xa = 0, ya = 0, za = 0, xb = 0, yb = 0, zb = 0;
    if (oka) chunk_cell(q, ch, l, xa, ya, za);
    if (okb) chunk_cell(q, ch, l + 1, xb, yb, zb);
    const Nbr oa = neighbours<L::D>(q, xa, ya, za), ob = neighbours<L::D>(q, xb, yb, zb);
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        unsigned va = 0u, vb = 0u;
        if (oka) va = __ldg(fin + ((unsigned)n * g.N + (unsigned)(ca + upstream<Q>(oa, n))));
        if (okb) vb = __ldg(fin + ((unsigned)n * g.N + (unsigned)(ca + 1 + upstream<Q>(ob, n))));
        v[n] = va | (vb << 16);
    }
}

template <int Q, class St, bool FORCED>
__global__ void __launch_bounds__(256, 3) k_batch_pair_pf(const typename St::T* __restrict__ fin_base,
                                                          typename St::T* __restrict__ fout_base,
                                                          const Chunk* __restrict__ chunks, int nchunks,
                                                          const KParams* __restrict__ dp,
                                                          const long long* __restrict__ offs) {
    const int G = gridDim.x;
    int ci = blockIdx.x;
    if (ci >= nchunks) return;
    unsigned cur[Q], nxt[Q];
    ChunkGeom gc = chunk_geom(chunks, dp, offs, ci);
    pair_load<Q, St>(fin_base, gc, cur);
    ChunkGeom gn = gc;
    if (ci + G < nchunks) gn = chunk_geom(chunks, dp, offs, ci + G);
    for (; ci < nchunks; ci += G) {
        const bool more = ci + G < nchunks;
        if (more) pair_load<Q, St>(fin_base, gn, nxt);
        ChunkGeom gnn = gn;
        if (ci + 2 * G < nchunks) gnn = chunk_geom(chunks, dp, offs, ci + 2 * G);
        // collide and store chunk ci
        const int dom = chunks[ci].dom;
        const KParams& p = dp[dom];
        typename St::T* fout = fout_base + gc.off;
        const int ca = gc.c0 + 2 * (int)threadIdx.x;
        const bool oka = ca < (int)gc.N, okb = ca + 1 < (int)gc.N;
        if (oka) {
            float2 g[Q];
#pragma unroll
            for (int n = 0; n < Q; ++n) g[n] = make_float2(St::dec1(cur[n] & 0xFFFFu), St::dec1(okb ? cur[n] >> 16 : cur[n] & 0xFFFFu));
            collide_shift<Q, A2, FORCED>(p, g);
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                const unsigned e = (unsigned)n * gc.N + (unsigned)ca;
                if (okb && (e & 1u) == 0) {
                    St::str2(fout, e, g[n]);
                } else {
                    St::str1(fout, e, g[n].x);
                    if (okb) St::str1(fout, e + 1, g[n].y);
                }
            }
        }
        if (more) {
#pragma unroll
            for (int n = 0; n < Q; ++n) cur[n] = nxt[n];
        }
        gc = gn;
        gn = gnn;
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
// prefetch (16-bit storages, K = 2, persistent): the prefetching kernel k_batch_pair_pf.
template <class St, int ARITH>
cudaError_t launch_batch_t(int q, bool forced, int K, bool persistent, const void* fin, void* fout,
                           const Chunk* chunks, int nchunks, const int2* walls, int nwalls, const KParams* dp,
                           const long long* offs, cudaStream_t s, bool prefetch = false) {
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
        else if (K == 2 && !(persistent && St::kShift && prefetch)) { MPH_BK(2) }
        else if (K == 2) {
            if constexpr (St::kShift) {
                auto kern = forced ? k_batch_pair_pf<Q, St, true> : k_batch_pair_pf<Q, St, false>;
                const int g = persistent_grid(kern);
                if (g <= 0) return cudaErrorInvalidConfiguration;
                kern<<<g < nchunks ? g : nchunks, 256, 0, s>>>(in, out, chunks, nchunks, dp, offs);
            }
        } else {
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
                     cudaStream_t s, bool prefetch);
MPH_DECL_BATCH(launch_batch_exact)
MPH_DECL_BATCH(launch_batch_fast_f64)
MPH_DECL_BATCH(launch_batch_f32)
MPH_DECL_BATCH(launch_batch_f16s)
MPH_DECL_BATCH(launch_batch_bf16s)
MPH_DECL_BATCH(launch_batch_f16c)
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
