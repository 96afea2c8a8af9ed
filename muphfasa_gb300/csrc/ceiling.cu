// ceiling.cu -- the memory pattern of the step without its arithmetic: a
// pull-stencil copy (every cell reads its Q populations from x - c_n, with
// the periodic wrap of the step kernels' index code, and writes them to its
// own slots), timed with CUDA events.  It measures what HBM delivers for the
// step's access pattern at each element size, the ceiling the step kernels'
// roofline fractions are read against.  No counterpart in the reference.
//
// Patterns (mode):
//   0  one cell per thread, one load per population (the 8- and 4-byte step
//      kernels);
//   1  two cells per thread for 2-byte elements, as k_step_pair: one 32-bit
//      word for a c_x = 0 population, two 16-bit loads for the others, 32-bit
//      stores;
//   2  two cells per thread for 2-byte elements, one aligned 32-bit word per
//      population: the x-shifted pair is assembled from the neighbouring
//      lane's word by a warp shuffle (lanes at a warp or row edge load the
//      missing 16-bit value), 32-bit stores.
#include <string>

#include "lbm_kernels.cuh"
#include "mph_internal.h"

namespace mph {
namespace {

template <int Q, class T>
__global__ void __launch_bounds__(256) k_copy_cells(const T* __restrict__ fin, T* __restrict__ fout, const KParams p) {
    using L = Lat<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= p.nx || y >= p.ny) return;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)(((long long)z * p.ny + y) * p.nx + x);
    const Nbr o = neighbours<L::D>(p, x, y, z);
#pragma unroll
    for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = __ldg(fin + ((unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n))));
}

template <int Q>
__global__ void __launch_bounds__(256) k_copy_pairs(const unsigned short* __restrict__ fin,
                                                     unsigned short* __restrict__ fout, const KParams p) {
    using L = Lat<Q>;
    const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= p.nx || y >= p.ny) return;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)(((long long)z * p.ny + y) * p.nx + x);
    const Nbr oa = neighbours<L::D>(p, x, y, z), ob = neighbours<L::D>(p, x + 1, y, z);
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const unsigned ea = (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(oa, n));
        unsigned w;
        if (L::cx(n) == 0) {
            w = __ldg(reinterpret_cast<const unsigned*>(fin + ea));
        } else {
            const unsigned eb = (unsigned)n * N + (unsigned)((int)ci + 1 + upstream<Q>(ob, n));
            w = (unsigned)__ldg(fin + ea) | ((unsigned)__ldg(fin + eb) << 16);
        }
        *reinterpret_cast<unsigned*>(fout + (unsigned)n * N + ci) = w;
    }
}

template <int Q>
__global__ void __launch_bounds__(256) k_copy_words(const unsigned short* __restrict__ fin,
                                                     unsigned short* __restrict__ fout, const KParams p) {
    using L = Lat<Q>;
    const int lane = threadIdx.x & 31;  // blockDim.x is a multiple of 32: a warp lies in one row
    const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool act = x < p.nx && y < p.ny;
    const unsigned N = (unsigned)p.ncell;
    const unsigned ci = act ? (unsigned)(((long long)z * p.ny + y) * p.nx + x) : 0u;
    const unsigned row = ci - (unsigned)x;  // first cell of the row
    const Nbr o = neighbours<L::D>(p, act ? x : 0, act ? y : 0, z);
    const int xl = x == 0 ? p.nx - 1 : x - 1;        // x - 1 with the periodic wrap
    const int xr = x + 2 >= p.nx ? x + 2 - p.nx : x + 2;  // x + 2 with the wrap
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const int oyz = (L::cy(n) == 1 ? o.ym : (L::cy(n) == -1 ? o.yp : 0)) +
                        (L::cz(n) == 1 ? o.zm : (L::cz(n) == -1 ? o.zp : 0));
        const unsigned base = (unsigned)n * N + (unsigned)((int)row + oyz);  // source row start
        const unsigned W = act ? __ldg(reinterpret_cast<const unsigned*>(fin + base + x)) : 0u;
        unsigned w = W;
        if (L::cx(n) == 1) {  // (x - 1, x): the previous lane's high half and this word's low half
            const unsigned P = __shfl_up_sync(0xffffffffu, W, 1);
            unsigned lo = P >> 16;
            if ((lane == 0 || x == 0) && act) lo = __ldg(fin + base + xl);
            w = lo | (W << 16);
        } else if (L::cx(n) == -1) {  // (x + 1, x + 2): this word's high half and the next lane's low half
            const unsigned Nw = __shfl_down_sync(0xffffffffu, W, 1);
            unsigned hi = Nw & 0xFFFFu;
            if ((lane == 31 || x + 2 >= p.nx) && act) hi = __ldg(fin + base + xr);
            w = (W >> 16) | (hi << 16);
        }
        if (act) *reinterpret_cast<unsigned*>(fout + (unsigned)n * N + ci) = w;
    }
}

// Instruction throughput of one pipe: every thread runs kIlp independent
// dependency chains of `iters` operations (enough independent work to fill
// the pipe), and the chains are folded into one stored value so nothing is
// dead code.
//   op 0 DFMA (FP64 pipe)   1 FFMA (FP32)   2 IMAD 32-bit   3 64-bit unsigned
//   high multiply + add (the fixed-point step's multiply)   4 int64 -> FP64
//   conversion + FP64 add (the conversions of fixed-point loads and stores)
constexpr int kIlp = 8;

template <int OP>
__global__ void __launch_bounds__(256) k_pipe(double* __restrict__ out, int iters, double a) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    double r = 0.0;
    if (OP == 0) {
        double x[kIlp];
        for (int i = 0; i < kIlp; ++i) x[i] = t * 1e-9 + i;
        for (int it = 0; it < iters; ++it)
#pragma unroll
            for (int i = 0; i < kIlp; ++i) x[i] = fma(x[i], a, 1e-3);
        for (int i = 0; i < kIlp; ++i) r += x[i];
    } else if (OP == 1) {
        float x[kIlp];
        const float af = (float)a;
        for (int i = 0; i < kIlp; ++i) x[i] = t * 1e-6f + i;
        for (int it = 0; it < iters; ++it)
#pragma unroll
            for (int i = 0; i < kIlp; ++i) x[i] = fmaf(x[i], af, 1e-3f);
        for (int i = 0; i < kIlp; ++i) r += x[i];
    } else if (OP == 2) {
        unsigned x[kIlp];
        const unsigned m = (unsigned)(a * 1e6) | 1u;
        for (int i = 0; i < kIlp; ++i) x[i] = t + i;
        for (int it = 0; it < iters; ++it)
#pragma unroll
            for (int i = 0; i < kIlp; ++i) x[i] = x[i] * m + 7u;
        unsigned s = 0;
        for (int i = 0; i < kIlp; ++i) s ^= x[i];
        r = s;
    } else if (OP == 3) {
        unsigned long long x[kIlp];
        const unsigned long long m = (unsigned long long)(a * 1e15) | 1ull;
        for (int i = 0; i < kIlp; ++i) x[i] = t * 0x9E3779B97F4A7C15ull + i;
        for (int it = 0; it < iters; ++it)
#pragma unroll
            for (int i = 0; i < kIlp; ++i) x[i] = __umul64hi(x[i], m) + x[i];
        unsigned long long s = 0;
        for (int i = 0; i < kIlp; ++i) s ^= x[i];
        r = (double)(s >> 11);
    } else {
        double x[kIlp];
        long long v[kIlp];
        for (int i = 0; i < kIlp; ++i) { x[i] = 0.0; v[i] = (long long)t * 3 + i; }
        for (int it = 0; it < iters; ++it)
#pragma unroll
            for (int i = 0; i < kIlp; ++i) {
                x[i] += (double)v[i];
                v[i] += it;
            }
        for (int i = 0; i < kIlp; ++i) r += x[i];
    }
    out[t] = r;
}

template <class F>
cudaError_t with_q3(int q, F&& f) {
    switch (q) {
        case 9: return f(std::integral_constant<int, 9>{});
        case 19: return f(std::integral_constant<int, 19>{});
        case 27: return f(std::integral_constant<int, 27>{});
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_copy(int elem, int mode, int q, const void* a, void* b, const KParams& p, cudaStream_t s) {
    return with_q3(q, [&](auto qc) -> cudaError_t {
        constexpr int Q = decltype(qc)::value;
        dim3 g, blk;
        auto shape = [&](int nxw, int threads) {
            int bx = ((nxw + 31) / 32) * 32;
            if (bx > threads) bx = threads;
            blk = dim3(bx, threads / bx, 1);
            g = dim3((nxw + bx - 1) / bx, (p.ny + blk.y - 1) / blk.y, p.nz);
        };
        if (mode == 0) {
            shape(p.nx, 256);
            if (elem == 8) k_copy_cells<Q, double><<<g, blk, 0, s>>>((const double*)a, (double*)b, p);
            else if (elem == 4) k_copy_cells<Q, float><<<g, blk, 0, s>>>((const float*)a, (float*)b, p);
            else k_copy_cells<Q, unsigned short><<<g, blk, 0, s>>>((const unsigned short*)a, (unsigned short*)b, p);
        } else if (mode == 1) {
            shape(p.nx / 2, 64);
            k_copy_pairs<Q><<<g, blk, 0, s>>>((const unsigned short*)a, (unsigned short*)b, p);
        } else {
            shape(p.nx / 2, 64);
            k_copy_words<Q><<<g, blk, 0, s>>>((const unsigned short*)a, (unsigned short*)b, p);
        }
        return cudaGetLastError();
    });
}

}  // namespace
}  // namespace mph

extern "C" int mph_pull_copy_timed(int elem_bytes, int mode, int q, int nx, int ny, int nz, int reps, float* ms) {
    using namespace mph;
    if (!ms || reps < 1 || nx < 2 || ny < 1 || nz < 1 || !(q == 9 || q == 19 || q == 27))
        return fail(MPH_ERR_ARG, "mph_pull_copy_timed: bad argument");
    if (!(elem_bytes == 8 || elem_bytes == 4 || elem_bytes == 2) || mode < 0 || mode > 2 ||
        (mode > 0 && (elem_bytes != 2 || nx % 2)) || (q == 9) != (nz == 1))
        return fail(MPH_ERR_ARG, "mph_pull_copy_timed: unsupported element size / pattern / lattice combination");
    const long long N = (long long)nx * ny * nz;
    if ((long long)q * N >= (1LL << 32) || ny > 65535 || nz > 65535)
        return fail(MPH_ERR_ARG, "mph_pull_copy_timed: grid too large");
    KParams p{};
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.periodic[0] = p.periodic[1] = p.periodic[2] = 1;
    p.ncell = N;
    p.y1 = ny;
    p.z1 = nz;
    const size_t bytes = (size_t)elem_bytes * q * N;
    void *a = nullptr, *b = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&a, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b, bytes);
    if (e == cudaSuccess) e = cudaMemset(a, 0, bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    for (int w = 0; w < 2 && e == cudaSuccess; ++w) e = launch_copy(elem_bytes, mode, q, w % 2 ? b : a, w % 2 ? a : b, p, s);
    if (e == cudaSuccess) e = cudaEventRecord(e0, s);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch_copy(elem_bytes, mode, q, r % 2 ? b : a, r % 2 ? a : b, p, s);
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(a);
    cudaFree(b);
    if (e != cudaSuccess) return fail(MPH_ERR_CUDA, std::string("mph_pull_copy_timed: ") + cudaGetErrorString(e));
    *ms = t / reps;
    return MPH_OK;
}

extern "C" int mph_pipe_rate(int op, double* ops_per_s) {
    using namespace mph;
    if (!ops_per_s || op < 0 || op > 4) return fail(MPH_ERR_ARG, "mph_pipe_rate: bad argument");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = 8 * sms, threads = 256, iters = 4096;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(double) * blocks * threads);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    auto launch = [&](int it) {
        switch (op) {
            case 0: k_pipe<0><<<blocks, threads>>>(out, it, 0.999999); break;
            case 1: k_pipe<1><<<blocks, threads>>>(out, it, 0.999999); break;
            case 2: k_pipe<2><<<blocks, threads>>>(out, it, 0.999999); break;
            case 3: k_pipe<3><<<blocks, threads>>>(out, it, 0.999999); break;
            default: k_pipe<4><<<blocks, threads>>>(out, it, 0.999999); break;
        }
        return cudaGetLastError();
    };
    if (e == cudaSuccess) e = launch(iters);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch(iters);
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return fail(MPH_ERR_CUDA, std::string("mph_pipe_rate: ") + cudaGetErrorString(e));
    *ops_per_s = 3.0 * blocks * threads * (double)iters * kIlp / (ms / 1e3);
    return MPH_OK;
}
