// k_f64_exact.cu -- kernels that follow the reference's floating-point
// operation order.  This translation unit is compiled with --fmad=false so
// that no multiply-add is contracted: together with IEEE division this makes
// the FP64 results bit-identical to the reference CPU path.
//
// Contents: the exact FP64 step; moments (updateMacroscopic), initial
// conditions (setInitialConditions), FP64 reductions and host<->storage
// conversions for every precision; and the plugin-level kernels on caller
// Array4 memory (pullCollideFusedArr, FillBoundary periodic copy, BCManager
// ghost fill).
#include <type_traits>

#include "batch_kernel.cuh"
#include "lbm_launch.h"
#include "mph.h"

namespace mph {

namespace {

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

template <class F>
cudaError_t with_store(int prec, F&& f) {
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

// Uploads report saturating stores into flag (weight-scaled 16-bit storage).
template <int Q, class St>
__global__ void __launch_bounds__(256) k_convert(typename St::T* __restrict__ store, double* __restrict__ f64, int n,
                                                 long long N, int to_store, int* flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (to_store) {
        unsigned sat = 0;
        st_chk<Q, St>(store, n, i, N, (typename St::R)f64[i], sat);
        report_to<St>(flag, sat);
    } else {
        f64[i] = (double)St::template ld<Q>(store, n, i, N);
    }
}

template <int Q, class St>
__global__ void __launch_bounds__(256) k_convert_slab(typename St::T* __restrict__ store, double* __restrict__ stage,
                                                      long long c0, long long cnt, long long N, int to_store,
                                                      int* flag) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cnt) return;
    const int n = blockIdx.y;
    double* v = stage + n * cnt + j;
    if (to_store) {
        unsigned sat = 0;
        st_chk<Q, St>(store, n, c0 + j, N, (typename St::R)*v, sat);
        report_to<St>(flag, sat);
    } else {
        *v = (double)St::template ld<Q>(store, n, c0 + j, N);
    }
}

__global__ void k_reduce_final(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
    // One warp per component, fixed order: deterministic.
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 4) return;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += part[4 * b + k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) out[k] = v;
}

// ---- plugin level: Array4 views on caller memory ------------------------
__device__ __forceinline__ double& at(const A4& a, int i, int j, int k, int n) {
    return a.p[(i - a.b[0]) + (long long)(j - a.b[1]) * a.js + (long long)(k - a.b[2]) * a.ks + (long long)n * a.ns];
}

// pullCollideFusedArr (Collision.cpp:18-92) over box lo..hi.
template <int Q, bool FORCED>
__global__ void __launch_bounds__(256) k_pull_collide_arr(A4 fin, A4 fout, int lo0, int lo1, int lo2, int nx, int ny,
                                                          const KParams p) {
    using L = Lat<Q>;
    const int i = lo0 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = lo1 + blockIdx.y * blockDim.y + threadIdx.y;
    const int k = lo2 + blockIdx.z;
    if (i >= lo0 + nx || j >= lo1 + ny) return;
    double f[Q];
#pragma unroll
    for (int n = 0; n < Q; ++n) f[n] = at(fin, i - L::cx(n), j - L::cy(n), k - L::cz(n), n);
    collide_exact<Q, FORCED>(p, f);
#pragma unroll
    for (int n = 0; n < Q; ++n) at(fout, i, j, k, n) = f[n];
}

__device__ __forceinline__ bool in_dom(const int* v, const int* dlo, const int* dhi, int D) {
    for (int d = 0; d < D; ++d)
        if (v[d] < dlo[d] || v[d] > dhi[d]) return false;
    return true;
}

struct Dom {
    int lo[3], hi[3], per[3];
};

// FillBoundary(periodicity) for one box covering the domain.
template <int Q>
__global__ void __launch_bounds__(256) k_periodic_fill_arr(A4 f, Dom dm) {
    using L = Lat<Q>;
    const long long nxg = f.e[0] - f.b[0], nyg = f.e[1] - f.b[1], nzg = f.e[2] - f.b[2];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nxg * nyg * nzg) return;
    int v[3] = {f.b[0] + (int)(t % nxg), f.b[1] + (int)((t / nxg) % nyg), f.b[2] + (int)(t / (nxg * nyg))};
    if (in_dom(v, dm.lo, dm.hi, L::D)) return;
    int img[3] = {v[0], v[1], v[2]};
    for (int d = 0; d < L::D; ++d) {
        if (v[d] < dm.lo[d] || v[d] > dm.hi[d]) {
            if (!dm.per[d]) return;
            const int len = dm.hi[d] - dm.lo[d] + 1;
            img[d] = (v[d] < dm.lo[d]) ? v[d] + len : v[d] - len;
        }
    }
    for (int d = 0; d < 3; ++d)
        if (img[d] < f.b[d] || img[d] >= f.e[d]) return;
    for (int n = 0; n < Q; ++n) at(f, v[0], v[1], v[2], n) = at(f, img[0], img[1], img[2], n);
}

// BCManager<L>::operator() (BoundaryConditions.H:124-189) on every ghost
// cell of f outside the domain, with the ghost-fill kernels of BCTypes/*.H.
template <int Q>
__global__ void __launch_bounds__(256) k_bc_fill_arr(A4 f, Dom dm, const KParams* __restrict__ pg) {
    using L = Lat<Q>;
    const long long nxg = f.e[0] - f.b[0], nyg = f.e[1] - f.b[1], nzg = f.e[2] - f.b[2];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nxg * nyg * nzg) return;
    int iv[3] = {f.b[0] + (int)(t % nxg), f.b[1] + (int)((t / nxg) % nyg), f.b[2] + (int)(t / (nxg * nyg))};
    if (in_dom(iv, dm.lo, dm.hi, L::D)) return;
    int code[3] = {0, 0, 0};
    for (int d = 0; d < L::D; ++d) {
        code[d] = iv[d] < dm.lo[d] ? -1 : (iv[d] > dm.hi[d] ? 1 : 0);
        if (dm.per[d]) code[d] = 0;
    }
    if (code[0] == 0 && code[1] == 0 && code[2] == 0) return;
    const int cls = (code[0] + 1) + 3 * (code[1] + 1) + (L::D == 3 ? 9 * (code[2] + 1) : 0);
    const int type = pg->bc_type[cls];
    if (type == kBcPeriodic) return;
    auto fab_has = [&](const int* s) {
        for (int d = 0; d < 3; ++d)
            if (s[d] < f.b[d] || s[d] >= f.e[d]) return false;
        return true;
    };
    for (int n = 0; n < Q; ++n) {
        const int src[3] = {iv[0] + L::cx(n), iv[1] + L::cy(n), iv[2] + L::cz(n)};
        if (!(in_dom(src, dm.lo, dm.hi, L::D) && fab_has(src))) continue;
        const int o = L::opp(n);
        if (type == kBcOutflow) {
            at(f, iv[0], iv[1], iv[2], n) = at(f, src[0], src[1], src[2], n);
        } else if (type == kBcPressure) {
            double rho = 0.0, j0 = 0.0, j1 = 0.0, j2 = 0.0;
            for (int m = 0; m < Q; ++m) {
                const double fm = at(f, src[0], src[1], src[2], m);
                rho += fm;
                j0 += L::cx(m) * fm;
                j1 += L::cy(m) * fm;
                if (L::D == 3) j2 += L::cz(m) * fm;
            }
            const double inv_rho = 1.0 / rho;
            double cu, uu;
            if (L::D == 2) {
                cu = (L::cx(n) * j0 + L::cy(n) * j1) * inv_rho;
                uu = (j0 * j0 + j1 * j1) * inv_rho * inv_rho;
            } else {
                cu = (L::cx(n) * j0 + L::cy(n) * j1 + L::cz(n) * j2) * inv_rho;
                uu = (j0 * j0 + j1 * j1 + j2 * j2) * inv_rho * inv_rho;
            }
            const double feq_even = L::w(n) * pg->bc_rho[cls] * (1.0 + 0.5 * cu * cu * 3.0 * 3.0 - 0.5 * uu * 3.0);
            at(f, iv[0], iv[1], iv[2], n) = -at(f, src[0], src[1], src[2], o) + 2.0 * feq_even;
        } else {
            double rho = 1;
            double U[3] = {0., 0., 0.};
            if (type != kBcNoSlip) {
                rho = pg->bc_rho[cls];
                U[0] = pg->bc_U[cls][0]; U[1] = pg->bc_U[cls][1]; U[2] = pg->bc_U[cls][2];
            }
            double cdotu;
            if (L::D == 2) cdotu = L::cx(o) * U[0] + L::cy(o) * U[1];
            else cdotu = L::cx(o) * U[0] + L::cy(o) * U[1] + L::cz(o) * U[2];
            const double contrib = -2. * rho * L::w(o) * cdotu * 3.0;
            at(f, iv[0], iv[1], iv[2], n) = at(f, src[0], src[1], src[2], o) + contrib;
        }
    }
}

}  // namespace

cudaError_t launch_step_exact(int q, bool forced, const double* fin, double* fout, const KParams& p,
                              const KParams* pg, cudaStream_t s) {
    dim3 g, b;
    step_shape(p, g, b);
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        if (forced) k_step<Q, StF64, kExact, true><<<g, b, 0, s>>>(fin, fout, p, pg);
        else k_step<Q, StF64, kExact, false><<<g, b, 0, s>>>(fin, fout, p, pg);
        return cudaGetLastError();
    });
}

cudaError_t launch_moments(int prec, int q, bool forced, const void* fin, double* rho, double* u, const KParams& p,
                           const KParams* pg, cudaStream_t s) {
    dim3 g, b;
    step_shape(p, g, b);
    return with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            auto in = static_cast<const typename St::T*>(fin);
            if (forced) k_moments<Q, St, true><<<g, b, 0, s>>>(in, rho, u, p, pg);
            else k_moments<Q, St, false><<<g, b, 0, s>>>(in, rho, u, p, pg);
            return cudaGetLastError();
        });
    });
}

cudaError_t launch_init(int prec, int q, bool forced, void* f, double* rho, double* u, const KParams& p,
                        cudaStream_t s) {
    dim3 g, b;
    flat_shape(p.ncell, g, b);
    return with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            auto out = static_cast<typename St::T*>(f);
            if (forced) k_init<Q, St, true><<<g, b, 0, s>>>(out, rho, u, p);
            else k_init<Q, St, false><<<g, b, 0, s>>>(out, rho, u, p);
            return cudaGetLastError();
        });
    });
}

cudaError_t launch_init_neq(int prec, int q, void* f, const double* rho, const double* u, const KParams& p,
                            cudaStream_t s) {
    dim3 g, b;
    flat_shape(p.ncell, g, b);
    return with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_init_neq<Q, St><<<g, b, 0, s>>>(static_cast<typename St::T*>(f), rho, u, p);
            return cudaGetLastError();
        });
    });
}

cudaError_t launch_reduce(int prec, int q, const void* f, long long ncell, double* part, int nblocks, double* out4,
                          cudaStream_t s) {
    cudaError_t e = with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_reduce_partial<Q, St><<<nblocks, 256, 0, s>>>(static_cast<const typename St::T*>(f), part, ncell);
            return cudaGetLastError();
        });
    });
    if (e != cudaSuccess) return e;
    k_reduce_final<<<1, 128, 0, s>>>(part, nblocks, out4);
    return cudaGetLastError();
}

cudaError_t launch_convert(int prec, int q, bool to_store, void* store, double* f64, int n, long long ncell,
                           cudaStream_t s, int* flag) {
    dim3 g, b;
    flat_shape(ncell, g, b);
    return with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_convert<Q, St><<<g, b, 0, s>>>(static_cast<typename St::T*>(store), f64, n, ncell, to_store ? 1 : 0,
                                             flag);
            return cudaGetLastError();
        });
    });
}

cudaError_t launch_convert_slab(int prec, int q, bool to_store, void* store, double* stage, long long c0,
                                long long cnt, long long ncell, cudaStream_t s, int* flag) {
    if (cnt <= 0) return cudaSuccess;
    const dim3 g((unsigned)((cnt + 255) / 256), (unsigned)q, 1), b(256, 1, 1);
    return with_store(prec, [&](auto st) {
        using St = decltype(st);
        return with_q(q, [&](auto qc) {
            constexpr int Q = decltype(qc)::value;
            k_convert_slab<Q, St><<<g, b, 0, s>>>(static_cast<typename St::T*>(store), stage, c0, cnt, ncell,
                                                  to_store ? 1 : 0, flag);
            return cudaGetLastError();
        });
    });
}

cudaError_t launch_pull_collide_arr(int dim, int q, bool forced, const int lo[3], const int hi[3], const A4& fin,
                                    const A4& fout, const KParams& p, cudaStream_t s) {
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = (dim == 3) ? hi[2] - lo[2] + 1 : 1;
    int bx = ((nx + 31) / 32) * 32;
    if (bx > 256) bx = 256;
    const int by = 256 / bx;
    dim3 b(bx, by, 1), g((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
    const int lo2 = (dim == 3) ? lo[2] : 0;
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        if (forced) k_pull_collide_arr<Q, true><<<g, b, 0, s>>>(fin, fout, lo[0], lo[1], lo2, nx, ny, p);
        else k_pull_collide_arr<Q, false><<<g, b, 0, s>>>(fin, fout, lo[0], lo[1], lo2, nx, ny, p);
        return cudaGetLastError();
    });
}

static Dom make_dom(int dim, const int dlo[3], const int dhi[3], const int per[3]) {
    Dom dm;
    for (int d = 0; d < 3; ++d) {
        dm.lo[d] = d < dim ? dlo[d] : 0;
        dm.hi[d] = d < dim ? dhi[d] : 0;
        dm.per[d] = d < dim ? per[d] : 0;
    }
    return dm;
}

cudaError_t launch_periodic_fill_arr(int dim, int q, const int dlo[3], const int dhi[3], const int per[3],
                                     const A4& f, cudaStream_t s) {
    const long long cells = (long long)(f.e[0] - f.b[0]) * (f.e[1] - f.b[1]) * (f.e[2] - f.b[2]);
    dim3 g, b;
    flat_shape(cells, g, b);
    const Dom dm = make_dom(dim, dlo, dhi, per);
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        k_periodic_fill_arr<Q><<<g, b, 0, s>>>(f, dm);
        return cudaGetLastError();
    });
}

cudaError_t launch_bc_fill_arr(int dim, int q, const int dlo[3], const int dhi[3], const int per[3],
                               const KParams* pg, const A4& f, cudaStream_t s) {
    const long long cells = (long long)(f.e[0] - f.b[0]) * (f.e[1] - f.b[1]) * (f.e[2] - f.b[2]);
    dim3 g, b;
    flat_shape(cells, g, b);
    const Dom dm = make_dom(dim, dlo, dhi, per);
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        k_bc_fill_arr<Q><<<g, b, 0, s>>>(f, dm, pg);
        return cudaGetLastError();
    });
}

cudaError_t launch_batch_exact(int q, bool forced, int K, bool persistent, const void* fin, void* fout, const Chunk* chunks, int nchunks,
                               const int2* walls, int nwalls, const KParams* dp, const long long* offs,
                               cudaStream_t s) {
    return launch_batch_t<StF64, kExact>(q, forced, K, persistent, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
}

}  // namespace mph
