// k_f64x_bulk.cu -- the FP64-accurate fixed-point step (MPH_PREC_F64X) with
// its pull operands staged in shared memory by one-dimensional bulk
// asynchronous copies (opt-in: MPH_F64X_KERNEL=bulk).
//
// The unit of work is a segment of kXB = 128 cells of one row (y, z) of the
// launch window, one cell per thread.  For population n the cells of a segment
// pull from one contiguous run of the SoA array: the segment shifted by
// (c_x, c_y, c_z), in the source row (y - c_y, z - c_z) wrapped across
// periodic faces.  Lane n of warp 0 computes that run (widened to 16-byte
// boundaries) and issues its cp.async.bulk copy into a ring of S shared-memory
// stages; the stage's mbarrier completes when all Q runs have landed, and a
// persistent block keeps S - 1 segments in flight while it collides the
// current one.  Pulls outside the staged runs (the x wrap at the row ends)
// read global memory, and cells next to a non-periodic face take pull_x's
// boundary rules, so every cell gets the values of k_step_x and the results
// are the same bits.  The per-cell work is collide_x (1300 instructions per
// D3Q19 cell), so the staging adds a few per cent of instructions while the
// loads leave the critical path.  Waits are bounded (bulk::bar_wait); on a
// timeout the block ORs 2 into *flag, waits (bounded) for its own copies and
// returns; a cell leaving the fixed-point range ORs 1, as in k_step_x.
#include "bulk_step.cuh"
#include "fx_kernels.cuh"
#include "lbm_launch.h"

namespace mph {

namespace {

constexpr int kXB = 128;          // cells per segment = threads per block
constexpr int kXLpad = kXB + 4;   // staged elements per run slot (the shift and the 16-byte widening)

struct XGeom {
    int cpr;         // segments per row
    int nchunks;     // segments of the window
    unsigned total;  // elements of the array, rounded down to a multiple of 2
};

template <int Q>
__device__ __forceinline__ void lane_cxyz(int n, int& cx, int& cy, int& cz) {
    cx = cy = cz = 0;
#pragma unroll
    for (int m = 0; m < Q; ++m)
        if (m == n) {
            cx = Lat<Q>::cx(m);
            cy = Lat<Q>::cy(m);
            cz = Lat<Q>::cz(m);
        }
}

// Warp 0: the Q runs of the segment [x0, x0 + len) of row (y, z) and their copies.
template <int Q>
__device__ __forceinline__ void issue_segment(const KParams& p, const i64* __restrict__ fin, int z, int y, int x0,
                                              int len, unsigned total, bulk::Run* rs, i64* dst,
                                              unsigned long long* b) {
    const int lane = threadIdx.x & 31;
    const unsigned N = (unsigned)p.ncell;
    bulk::Run run{0u, 0u};
    if (lane < Q) {
        int cx, cy, cz;
        lane_cxyz<Q>(lane, cx, cy, cz);
        int ys = y - cy, zs = z - cz;
        bool ok = true;
        if (ys < 0 || ys >= p.ny) {
            if (p.periodic[1]) ys = ys < 0 ? ys + p.ny : ys - p.ny;
            else ok = false;
        }
        if (zs < 0 || zs >= p.nz) {
            if (p.periodic[2]) zs = zs < 0 ? zs + p.nz : zs - p.nz;
            else ok = false;
        }
        const int xa = max(x0 - cx, 0), xe = min(x0 + len - cx, p.nx);
        if (ok && xe > xa) {
            const unsigned row = (unsigned)lane * N + (unsigned)((zs * p.ny + ys) * p.nx);
            unsigned e = (row + (unsigned)xe + 1u) & ~1u;
            if (e > total) e = total;
            run.base = (row + (unsigned)xa) & ~1u;
            run.len = e > run.base ? e - run.base : 0u;
        }
        rs[lane] = run;
    }
    unsigned bytes = 8u * run.len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
    __syncwarp();
    if (lane == 0) bulk::bar_expect(b, bytes);
    __syncwarp();
    if (lane < Q && run.len) bulk::copy_g2s(dst + (size_t)lane * kXLpad, fin + run.base, 8u * run.len, b);
}

template <int Q, bool FORCED, int S>
__global__ void __launch_bounds__(kXB, 4) k_step_x_bulk(const i64* __restrict__ fin, i64* __restrict__ fout,
                                                        const KParams p, const KParamsX px,
                                                        const KParams* __restrict__ pg, const i64* __restrict__ kbb,
                                                        const XGeom gm, int* __restrict__ flag) {
    using L = Lat<Q>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem);
    bulk::Run* runs = reinterpret_cast<bulk::Run*>(smem + 64);           // [S][Q]
    i64* data = reinterpret_cast<i64*>(smem + bulk::kHeader);            // [S][Q][kXLpad]
    const int tid = threadIdx.x;
    const unsigned N = (unsigned)p.ncell;
    const int G = gridDim.x, wy = p.y1 - p.y0;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) bulk::bar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto where = [&](int k, int& z, int& y, int& x0, int& len) {
        const int rr = k / gm.cpr;
        x0 = (k - rr * gm.cpr) * kXB;
        len = min(kXB, p.nx - x0);
        const int rz = rr / wy;
        y = p.y0 + (rr - rz * wy);
        z = p.z0 + rz;
    };
    auto issue = [&](int k, int s) {  // warp 0
        int z, y, x0, len;
        where(k, z, y, x0, len);
        issue_segment<Q>(p, fin, z, y, x0, len, gm.total, runs + s * Q, data + (size_t)s * Q * kXLpad, &bar[s]);
    };
    if (tid < 32)
        for (int i = 0; i < S - 1; ++i) {
            const int k = blockIdx.x + i * G;
            if (k < gm.nchunks) issue(k, i);
        }
    int it = 0, bad = 0;
    bool timed_out = false;
    for (int k = blockIdx.x; k < gm.nchunks; k += G, ++it) {
        const int s = it % S;
        const bool got = bulk::bar_wait(&bar[s], (unsigned)(it / S) & 1u);
        if (__syncthreads_or(!got)) {
            timed_out = true;
            break;
        }
        if (tid < 32) {
            const int kn = k + (S - 1) * G;
            if (kn < gm.nchunks) issue(kn, (it + S - 1) % S);
        }
        int z, y, x0, len;
        where(k, z, y, x0, len);
        if (tid < len) {
            const int x = x0 + tid;
            const long long c = ((long long)z * p.ny + y) * p.nx + x;
            const unsigned ci = (unsigned)c;
            const Nbr o = neighbours<L::D>(p, x, y, z);
            i64 h[Q];
            if (!o.wall) {
                const bulk::Run* rs = runs + s * Q;
                const i64* st = data + (size_t)s * Q * kXLpad;
#pragma unroll
                for (int n = 0; n < Q; ++n) {
                    const bulk::Run rn = rs[n];
                    const unsigned e = (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n));
                    const unsigned d = e - rn.base;
                    h[n] = d < rn.len ? st[(size_t)n * kXLpad + d] : __ldg(fin + e);
                }
            } else {
                pull_x<Q, false>(p, pg, kbb, fin, x, y, z, c, h);
            }
            collide_x<Q, FORCED>(px, h, bad);
#pragma unroll
            for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = h[n];
        }
        __syncthreads();
    }
    if (bad) atomicOr(flag, 1);
    if (timed_out) {
        if (tid == 0) {
            atomicOr(flag, 2);
            for (int i = 0; i < S - 1; ++i) {  // copies still in flight: iterations it .. it + S - 2
                const int j = it + i;
                if (blockIdx.x + j * G < gm.nchunks) bulk::bar_wait(&bar[j % S], (unsigned)(j / S) & 1u);
            }
        }
        __syncthreads();
    }
}

}  // namespace

// mode 0: raise the kernels' shared-memory limit (once per handle, before any
// launch or capture); mode 1: one step over the window of p.
// cudaErrorNotSupported where the kernel does not apply (obstacles, more
// elements than 32-bit indices cover, a stage count other than 2 or 3).
cudaError_t launch_step_f64x_bulk(int mode, int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                                  const KParamsX& px, const KParams* pg, const long long* kbb, int* flag, int stages,
                                  cudaStream_t s) {
    if (p.cls || stages < 2 || stages > 3) return cudaErrorNotSupported;
    const long long total = (long long)q * p.ncell;
    if (total >= (1LL << 32) - 64) return cudaErrorNotSupported;
    if ((reinterpret_cast<unsigned long long>(fin) | reinterpret_cast<unsigned long long>(fout)) & 15)
        return cudaErrorNotSupported;
    XGeom gm;
    gm.cpr = (p.nx + kXB - 1) / kXB;
    const long long nch = (long long)gm.cpr * (p.y1 - p.y0) * (p.z1 - p.z0);
    if (nch <= 0 || nch > 0x7fffffffLL) return cudaErrorNotSupported;
    gm.nchunks = (int)nch;
    gm.total = (unsigned)(total & ~1LL);
    const size_t smem = (size_t)bulk::kHeader + (size_t)stages * q * kXLpad * sizeof(long long);
    cudaError_t err = cudaErrorNotSupported;
    auto go = [&](auto kern) {
        if (mode == 0) {
            err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            return;
        }
        int dev = 0, sms = 0, per_sm = 0;
        err = cudaGetDevice(&dev);
        if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (err == cudaSuccess) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kXB, smem);
        if (err != cudaSuccess) return;
        int grid = per_sm * sms;
        if (grid <= 0) {
            err = cudaErrorInvalidConfiguration;
            return;
        }
        if (grid > gm.nchunks) grid = gm.nchunks;
        kern<<<grid, kXB, smem, s>>>(fin, fout, p, px, pg, kbb, gm, flag);
        err = cudaGetLastError();
    };
    auto pick = [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        if (stages == 2) {
            if (forced) go(k_step_x_bulk<Q, true, 2>);
            else go(k_step_x_bulk<Q, false, 2>);
        } else {
            if (forced) go(k_step_x_bulk<Q, true, 3>);
            else go(k_step_x_bulk<Q, false, 3>);
        }
        return err;
    };
    switch (q) {
        case 9: return pick(std::integral_constant<int, 9>{});
        case 15: return pick(std::integral_constant<int, 15>{});
        case 19: return pick(std::integral_constant<int, 19>{});
        case 27: return pick(std::integral_constant<int, 27>{});
    }
    return cudaErrorNotSupported;
}

}  // namespace mph
