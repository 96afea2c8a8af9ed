// bulk_step.cuh -- the 16-bit pair step (shifted FP16 / BF16 / 1-4-11
// storage) with its pull operands staged in shared memory by one-dimensional
// bulk asynchronous copies.  Included by the k_fast_* translation units of
// the 16-bit precisions.
//
// Why it exists: a 2-byte population gives a warp only 64 bytes per load
// instruction, so a direct pull keeps few bytes in flight (the measured copy
// ceiling of the pair pattern is 0.87-0.89 of the copy peak, the direct step
// reaches 0.72).  Measured on the 512^3 D3Q19 channel (FP16): 44 GLUPS (0.50)
// against the direct kernel's 63 (0.72).  An ncu capture at 256^3 shows why:
// the direct step is already close to issue-bound (357 instructions per cell,
// issue slots 56 % busy) and staging adds 46 % instructions (shared-memory
// loads, run bounds checks) plus block-barrier stalls.  The kernel is kept as
// an opt-in (MPH_PAIR_KERNEL=bulk; batches: MPH_BATCH_CANDIDATE=6), bit-
// identical to the direct one.  Here the unit of work is
// a chunk of whole rows (y, z) of the launch window.  For every population n
// the rows its cells pull from are the chunk's rows shifted by (c_y, c_z):
// one contiguous run of the population's SoA array (the x shift, periodic x
// wrap included, stays inside a row).  One thread issues Q cp.async.bulk
// copies of those runs into one stage of a ring of S shared-memory stages,
// all completing on that stage's mbarrier; a persistent block keeps S - 1
// chunks in flight while its 256 threads collide the current chunk from
// shared memory, one cell pair per thread at a time, and store to global
// memory directly (no registers hold data in flight).
//
// Pulls that fall outside the staged runs (rows wrapped by a periodic y or z
// face) read global memory, and pairs next to a non-periodic face take the
// boundary rules of the direct kernel: the values and the collide are those
// of k_step_pair, so the results are equal bit for bit.
//
// Alignment: a bulk copy moves a multiple of 16 bytes between 16-byte aligned
// addresses, so each run is widened to 8-element boundaries and clipped to the
// last whole 16 bytes of the array (anything past that is read directly).
// Waits: every mbarrier wait is bounded by %globaltimer; on a timeout the
// block ORs 2 into *flag, waits (bounded) for its copies still in flight and
// returns, so the context stays usable and the host reports the error.
#pragma once

#include "batch_kernel.cuh"
#include "lbm_kernels.cuh"

namespace mph {

// Launch geometry of one window, computed on the host.
struct BulkGeom {
    int rows;        // rows per chunk
    int cpp;         // chunks per plane of the window
    int nchunks;     // chunks of the window
    int lpad;        // elements of one staged run slot (a multiple of 8)
    unsigned total;  // elements of the array, rounded down to a multiple of 8
};

namespace bulk {

constexpr int kThreads = 256;
constexpr int kHeader = 1024;  // bytes before the staged data: mbarriers and run table
constexpr unsigned long long kWaitNs = 200ull * 1000 * 1000;
constexpr unsigned long long kSpinLimit = 1ull << 26;

struct Run {
    unsigned base;  // element index of the staged run in the array
    unsigned len;   // staged elements (0: nothing staged)
};

__device__ __forceinline__ unsigned sa(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

__device__ __forceinline__ void bar_init(unsigned long long* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(sa(b)) : "memory");
}

// The one arrival of a phase, announcing `bytes` of copies that complete it.
__device__ __forceinline__ void bar_expect(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sa(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* b) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(sa(dst)),
        "l"(src), "r"(bytes), "r"(sa(b))
        : "memory");
}

// Bounded wait for the phase of parity `parity`; false on timeout.
__device__ __forceinline__ bool bar_wait(unsigned long long* b, unsigned parity) {
    const unsigned addr = sa(b);
    const unsigned long long t0 = now_ns();
    for (unsigned long long it = 0; it < kSpinLimit; ++it) {
        unsigned done;
        asm volatile(
            "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\nselp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63 && now_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

// (c_y, c_z) of population n for a runtime n, by compile-time selects (an
// indexed lattice table would live in local memory).
template <int Q>
__device__ __forceinline__ void lane_c(int n, int& cy, int& cz) {
    cy = 0;
    cz = 0;
#pragma unroll
    for (int m = 0; m < Q; ++m)
        if (m == n) {
            cy = Lat<Q>::cy(m);
            cz = Lat<Q>::cz(m);
        }
}

// Warp 0, lane n < Q: the staged run of population n for rows [yb, yb + r) of
// plane z (in the array's element indices, widened to 8-element boundaries
// and clipped at `total`); lane 0 announces the stage's bytes on its mbarrier
// and every lane with a run issues its copy.
template <int Q, class T>
__device__ __forceinline__ void issue_runs(const KParams& p, const T* __restrict__ fin, int z, int yb, int r,
                                           unsigned total, Run* rs, unsigned short* dst, int lpad,
                                           unsigned long long* b) {
    const int lane = threadIdx.x & 31;
    const unsigned N = (unsigned)p.ncell;
    Run run{0u, 0u};
    if (lane < Q) {
        int cy, cz;
        lane_c<Q>(lane, cy, cz);
        int zs = z - cz;
        bool ok = true;
        if (zs < 0 || zs >= p.nz) {
            if (p.periodic[2]) zs = zs < 0 ? zs + p.nz : zs - p.nz;
            else ok = false;
        }
        const int ya = max(yb - cy, 0), ye = min(yb + r - cy, p.ny);
        if (ok && ye > ya) {
            const unsigned a = (unsigned)lane * N + (unsigned)((zs * p.ny + ya) * p.nx);
            const unsigned e0 = (unsigned)lane * N + (unsigned)((zs * p.ny + ye) * p.nx);
            unsigned e = (e0 + 7u) & ~7u;
            if (e > total) e = total;
            run.base = a & ~7u;
            run.len = e > run.base ? e - run.base : 0u;
        }
        rs[lane] = run;
    }
    unsigned bytes = 2u * run.len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
    __syncwarp();
    if (lane == 0) bar_expect(b, bytes);
    __syncwarp();
    if (lane < Q && run.len) copy_g2s(dst + (size_t)lane * lpad, fin + run.base, 2u * run.len, b);
}

}  // namespace bulk

template <int Q, class St, bool FORCED, int S>
__global__ void __launch_bounds__(bulk::kThreads, 3) k_step_pair_bulk(const typename St::T* __restrict__ fin,
                                                                   typename St::T* __restrict__ fout, const KParams p,
                                                                   const KParams* __restrict__ pg, const BulkGeom gm,
                                                                   int* __restrict__ flag) {
    using L = Lat<Q>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
    bulk::Run* runs = reinterpret_cast<bulk::Run*>(smem + 64);  // [S][Q]
    unsigned short* data = reinterpret_cast<unsigned short*>(smem + bulk::kHeader);  // [S][Q][lpad]
    const int tid = threadIdx.x;
    const unsigned N = (unsigned)p.ncell;
    const int G = gridDim.x;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) bulk::bar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    // Warp 0: the runs of chunk k into stage s, and their copies.
    auto issue = [&](int k, int s) {
        const int pz = k / gm.cpp;
        const int yb = p.y0 + (k - pz * gm.cpp) * gm.rows;
        bulk::issue_runs<Q>(p, fin, p.z0 + pz, yb, min(gm.rows, p.y1 - yb), gm.total, runs + s * Q,
                            data + (size_t)s * Q * gm.lpad, gm.lpad, &bar[s]);
    };

    if (tid < 32)
        for (int i = 0; i < S - 1; ++i) {
            const int k = blockIdx.x + i * G;
            if (k < gm.nchunks) issue(k, i);
        }
    int it = 0;
    bool timed_out = false;
    for (int k = blockIdx.x; k < gm.nchunks; k += G, ++it) {
        const int s = it % S;
        const bool got = bulk::bar_wait(&bar[s], (unsigned)(it / S) & 1u);
        if (__syncthreads_or(!got)) {
            timed_out = true;
            break;
        }
        // Warp 0 refills the stage consumed in the previous iteration (every
        // thread passed that iteration's closing barrier) with the chunk S - 1
        // ahead, while the other warps start on this chunk.
        if (tid < 32) {
            const int kn = k + (S - 1) * G;
            if (kn < gm.nchunks) issue(kn, (it + S - 1) % S);
        }
        const bulk::Run* rs = runs + s * Q;
        const unsigned short* st = data + (size_t)s * Q * gm.lpad;
        const int pz = k / gm.cpp;
        const int z = p.z0 + pz;
        const int yb = p.y0 + (k - pz * gm.cpp) * gm.rows;
        const int r = min(gm.rows, p.y1 - yb);
        const int hx = p.nx >> 1;
        const int npairs = r * hx;
#pragma unroll 1
        for (int j = tid; j < npairs; j += bulk::kThreads) {
            const int row = j / hx;
            const int x = 2 * (j - row * hx);
            const int y = yb + row;
            const unsigned ci = (unsigned)(((long long)z * p.ny + y) * p.nx + x);
            const Nbr oa = neighbours<L::D>(p, x, y, z), ob = neighbours<L::D>(p, x + 1, y, z);
            float2 g[Q];
            if (!oa.wall && !ob.wall) {
#pragma unroll
                for (int n = 0; n < Q; ++n) {
                    const bulk::Run rn = rs[n];
                    const unsigned ea = (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(oa, n));
                    const unsigned da = ea - rn.base;
                    const unsigned short* sn = st + (size_t)n * gm.lpad;
                    if (L::cx(n) == 0) {
                        // ea is even and run bases are multiples of 8: an aligned word
                        g[n] = da < rn.len ? St::dec2(*reinterpret_cast<const unsigned*>(sn + da)) : St::ldr2(fin, ea);
                    } else {
                        const unsigned eb = (unsigned)n * N + (unsigned)((int)ci + 1 + upstream<Q>(ob, n));
                        const unsigned db = eb - rn.base;
                        const float va = da < rn.len ? St::dec1(sn[da]) : St::ldr1(fin, ea);
                        const float vb = db < rn.len ? St::dec1(sn[db]) : St::ldr1(fin, eb);
                        g[n] = make_float2(va, vb);
                    }
                }
            } else {
                float ga[Q], gb[Q];
                pull_shift<Q, St>(p, pg, fin, x, y, z, ci, ga);
                pull_shift<Q, St>(p, pg, fin, x + 1, y, z, ci + 1, gb);
#pragma unroll
                for (int n = 0; n < Q; ++n) g[n] = make_float2(ga[n], gb[n]);
            }
            collide_shift<Q, A2, FORCED>(p, g);
#pragma unroll
            for (int n = 0; n < Q; ++n) St::str2(fout, (unsigned)n * N + ci, g[n]);
        }
        __syncthreads();
    }
    if (timed_out) {
        if (tid == 0) {
            atomicOr(flag, 2);
            // copies still in flight: the chunks of iterations it .. it + S - 2
            for (int i = 0; i < S - 1; ++i) {
                const int j = it + i;
                if (blockIdx.x + j * G < gm.nchunks) bulk::bar_wait(&bar[j % S], (unsigned)(j / S) & 1u);
            }
        }
        __syncthreads();
    }
}

// Shared-memory bytes of a launch with `stages` stages of Q runs of lpad elements.
inline size_t bulk_smem_bytes(int q, int stages, int lpad) {
    return (size_t)bulk::kHeader + (size_t)stages * q * lpad * 2;
}

// Geometry of the window of p with chunks of about `cells` cells (whole rows;
// at least one row).  Returns false when the launch does not apply: odd nx,
// obstacles, a run slot too large for shared memory, or more elements than
// the 32-bit element indices cover.
constexpr int kBulkMaxSmem = 227 * 1024;

inline bool bulk_geometry(const KParams& p, int q, int stages, int cells, long long total_elems, BulkGeom& gm) {
    if (p.nx % 2 != 0 || p.cls || stages < 2 || stages > 3) return false;
    if (total_elems >= (1LL << 32) - 64) return false;
    int rows = cells / p.nx;
    if (rows < 1) rows = 1;
    const int wy = p.y1 - p.y0;
    if (rows > wy) rows = wy;
    if (rows < 1) return false;
    gm.rows = rows;
    gm.cpp = (wy + rows - 1) / rows;
    const long long nch = (long long)gm.cpp * (p.z1 - p.z0);
    if (nch <= 0 || nch > 0x7fffffffLL) return false;
    gm.nchunks = (int)nch;
    gm.lpad = ((rows * p.nx + 14) + 7) & ~7;
    gm.total = (unsigned)(total_elems & ~7LL);
    return bulk_smem_bytes(q, stages, gm.lpad) <= (size_t)kBulkMaxSmem;
}

// Resident blocks of the kernel with `smem` dynamic shared memory times the
// SM count (host-side queries only, so a launch under stream capture may
// call it); 0 on error.
template <class Kern>
int bulk_grid(Kern k, size_t smem) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, bulk::kThreads, smem) != cudaSuccess) return 0;
    return per_sm * sms;
}

// mode 0: raise the dynamic shared-memory limit of the kernels of (q,
// forced, stages) to the largest block allowance (once per handle, before
// any launch or capture); mode 1: launch one step.  cudaErrorNotSupported
// when the launch does not apply to this window (the caller steps it with
// the direct kernel).
template <class St>
cudaError_t launch_step_bulk_t(int mode, int q, bool forced, const void* fin, void* fout, const KParams& p,
                               const KParams* pg, long long total_elems, int cells, int stages, int* flag,
                               cudaStream_t s) {
    BulkGeom gm;
    size_t smem = 0;
    if (mode == 1) {
        if (!bulk_geometry(p, q, stages, cells, total_elems, gm)) return cudaErrorNotSupported;
        if ((reinterpret_cast<unsigned long long>(fin) | reinterpret_cast<unsigned long long>(fout)) & 15)
            return cudaErrorNotSupported;
        smem = bulk_smem_bytes(q, stages, gm.lpad);
    }
    auto in = static_cast<const typename St::T*>(fin);
    auto out = static_cast<typename St::T*>(fout);
    cudaError_t err = cudaErrorInvalidValue;
    auto go = [&](auto kern) {
        if (mode == 0) {
            err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kBulkMaxSmem);
            return;
        }
        int grid = bulk_grid(kern, smem);
        if (grid <= 0) {
            err = cudaGetLastError();
            if (err == cudaSuccess) err = cudaErrorInvalidConfiguration;
            return;
        }
        if (grid > gm.nchunks) grid = gm.nchunks;
        kern<<<grid, bulk::kThreads, smem, s>>>(in, out, p, pg, gm, flag);
        err = cudaGetLastError();
    };
#define MPH_BULK_S(QQ, SS)                                      \
    if (stages == SS) {                                         \
        if (forced) go(k_step_pair_bulk<QQ, St, true, SS>);     \
        else go(k_step_pair_bulk<QQ, St, false, SS>);           \
        return err;                                             \
    }
#define MPH_BULK_Q(QQ)    \
    case QQ:              \
        MPH_BULK_S(QQ, 2) \
        MPH_BULK_S(QQ, 3) \
        return cudaErrorNotSupported;
    switch (q) {
        MPH_BULK_Q(9)
        MPH_BULK_Q(15)
        MPH_BULK_Q(19)
        MPH_BULK_Q(27)
    }
#undef MPH_BULK_Q
#undef MPH_BULK_S
    return cudaErrorNotSupported;
}

// ---- batches ------------------------------------------------------------
// The same staging over a batch of domains of any sizes (the batch's chunk
// kernel: every cell pulls through the wrapped neighbour offsets, and the
// cells next to non-periodic faces or obstacles are recomputed afterwards by
// k_batch_walls from the wall list, so pairs whose two cells are both on a
// face are skipped here).  Pairs are consecutive cells of the chunk (they may
// straddle two rows when nx is odd); every value is read as 16 bits, from the
// staged runs or, outside them, from global memory.  Domains start on
// 128-element boundaries and their runs are clipped to the domain's
// allocation, rounded up to 8 elements.
template <int Q, class St, bool FORCED, int S>
__global__ void __launch_bounds__(bulk::kThreads, 3) k_batch_pair_bulk(const typename St::T* __restrict__ fin_base,
                                                                    typename St::T* __restrict__ fout_base,
                                                                    const RowChunk* __restrict__ chunks, int nchunks,
                                                                    const KParams* __restrict__ dp,
                                                                    const long long* __restrict__ offs, int lpad,
                                                                    int* __restrict__ flag) {
    using L = Lat<Q>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
    bulk::Run* runs = reinterpret_cast<bulk::Run*>(smem + 64);
    unsigned short* data = reinterpret_cast<unsigned short*>(smem + bulk::kHeader);
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) bulk::bar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](int k, int s) {  // warp 0
        const RowChunk ch = chunks[k];
        const KParams& p = dp[ch.dom];
        const unsigned total = ((unsigned)Q * (unsigned)p.ncell + 7u) & ~7u;
        bulk::issue_runs<Q>(p, fin_base + offs[ch.dom], ch.z, ch.yb, ch.r, total, runs + s * Q,
                            data + (size_t)s * Q * lpad, lpad, &bar[s]);
    };

    if (tid < 32)
        for (int i = 0; i < S - 1; ++i) {
            const int k = blockIdx.x + i * G;
            if (k < nchunks) issue(k, i);
        }
    int it = 0;
    bool timed_out = false;
    for (int k = blockIdx.x; k < nchunks; k += G, ++it) {
        const int s = it % S;
        const bool got = bulk::bar_wait(&bar[s], (unsigned)(it / S) & 1u);
        if (__syncthreads_or(!got)) {
            timed_out = true;
            break;
        }
        if (tid < 32) {
            const int kn = k + (S - 1) * G;
            if (kn < nchunks) issue(kn, (it + S - 1) % S);
        }
        const RowChunk ch = chunks[k];
        const KParams& p = dp[ch.dom];
        const long long off = offs[ch.dom];
        const typename St::T* fin = fin_base + off;
        typename St::T* fout = fout_base + off;
        const unsigned N = (unsigned)p.ncell;
        const bulk::Run* rs = runs + s * Q;
        const unsigned short* st = data + (size_t)s * Q * lpad;
        const int ncells = ch.r * p.nx;
        const unsigned c0 = (unsigned)((ch.z * p.ny + ch.yb) * p.nx);
#pragma unroll 1
        for (int j = tid; 2 * j < ncells; j += bulk::kThreads) {
            const int la = 2 * j;
            const bool okb = la + 1 < ncells;
            const int ra = la / p.nx, xa = la - ra * p.nx;
            const int lb = okb ? la + 1 : la;
            const int rb = lb / p.nx, xb = lb - rb * p.nx;
            const Nbr oa = neighbours<L::D>(p, xa, ch.yb + ra, ch.z);
            const Nbr ob = neighbours<L::D>(p, xb, ch.yb + rb, ch.z);
            if (oa.wall && ob.wall) continue;  // both recomputed by the wall-list kernel
            const unsigned ca = c0 + (unsigned)la, cb = c0 + (unsigned)lb;
            float2 g[Q];
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                const bulk::Run rn = rs[n];
                const unsigned short* sn = st + (size_t)n * lpad;
                const unsigned ea = (unsigned)n * N + (unsigned)((int)ca + upstream<Q>(oa, n));
                const unsigned eb = (unsigned)n * N + (unsigned)((int)cb + upstream<Q>(ob, n));
                const unsigned da = ea - rn.base, db = eb - rn.base;
                const float va = da < rn.len ? St::dec1(sn[da]) : St::ldr1(fin, ea);
                const float vb = db < rn.len ? St::dec1(sn[db]) : St::ldr1(fin, eb);
                g[n] = make_float2(va, vb);
            }
            collide_shift<Q, A2, FORCED>(p, g);
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                const unsigned e = (unsigned)n * N + ca;
                if (okb && (e & 1u) == 0) {
                    St::str2(fout, e, g[n]);
                } else {
                    St::str1(fout, e, g[n].x);
                    if (okb) St::str1(fout, e + 1, g[n].y);
                }
            }
        }
        __syncthreads();
    }
    if (timed_out) {
        if (tid == 0) {
            atomicOr(flag, 2);
            for (int i = 0; i < S - 1; ++i) {
                const int j = it + i;
                if (blockIdx.x + j * G < nchunks) bulk::bar_wait(&bar[j % S], (unsigned)(j / S) & 1u);
            }
        }
        __syncthreads();
    }
}

// mode 0: raise the dynamic shared-memory limit (once per batch, before any
// launch or capture); mode 1: one batch step (the staged chunk kernel, then
// the wall cells).
template <class St>
cudaError_t launch_batch_bulk_t(int mode, int q, bool forced, int stages, int lpad, const void* fin, void* fout,
                                const RowChunk* chunks, int nchunks, const int2* walls, int nwalls,
                                const KParams* dp, const long long* offs, int* flag, cudaStream_t s) {
    const size_t smem = bulk_smem_bytes(q, stages, lpad);
    if (smem > (size_t)kBulkMaxSmem) return cudaErrorNotSupported;
    auto in = static_cast<const typename St::T*>(fin);
    auto out = static_cast<typename St::T*>(fout);
    cudaError_t err = cudaErrorNotSupported;
    auto go = [&](auto kern) {
        if (mode == 0) {
            err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kBulkMaxSmem);
            return;
        }
        int grid = bulk_grid(kern, smem);
        if (grid <= 0) {
            err = cudaGetLastError();
            if (err == cudaSuccess) err = cudaErrorInvalidConfiguration;
            return;
        }
        if (grid > nchunks) grid = nchunks;
        kern<<<grid, bulk::kThreads, smem, s>>>(in, out, chunks, nchunks, dp, offs, lpad, flag);
        err = cudaGetLastError();
    };
    return batch_with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        if (stages == 2) {
            if (forced) go(k_batch_pair_bulk<Q, St, true, 2>);
            else go(k_batch_pair_bulk<Q, St, false, 2>);
        } else if (stages == 3) {
            if (forced) go(k_batch_pair_bulk<Q, St, true, 3>);
            else go(k_batch_pair_bulk<Q, St, false, 3>);
        } else {
            return cudaErrorNotSupported;
        }
        if (err != cudaSuccess || mode == 0) return err;
        if (nwalls > 0) {
            const int nb = (nwalls + 255) / 256;
            if (forced) k_batch_walls<Q, St, kFast, true><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, offs);
            else k_batch_walls<Q, St, kFast, false><<<nb, 256, 0, s>>>(in, out, walls, nwalls, dp, offs);
        }
        return cudaGetLastError();
    });
}

}  // namespace mph
