// bench_probes.cu -- throughput probes of the GB300 pipes and of the pull-stencil
// memory pattern, used to explain the step kernels' rooflines:
//   FP64 (DFMA/DADD/DDIV), FP32 FFMA, INT32 IMAD, 64-bit high multiplies,
//   int64<->double and int32->float conversions, a plain copy, and a
//   19-population pull-copy (the step's memory traffic without its arithmetic),
//   and the host link (page-locked copies each way and both at once).
// Build and run: python bench.py --probes   (nvcc -O3 -gencode arch=compute_103a,code=sm_103a)
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("CUDA %s at %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

constexpr int ILP = 8;

__global__ void k_dfma(double* out, int iters, double a, double b) {
    double x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = fma(x[i], a, b);
    double s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_dadd(double* out, int iters, double a, double b) {
    double x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = __dadd_rn(x[i], a);
    double s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s + b;
}
__global__ void k_ddiv(double* out, int iters, double a, double b) {
    double x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3 + i + 1.0;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = a / x[i] + b;
    double s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_ffma(double* out, int iters, double a_, double b_) {
    float a = (float)a_, b = (float)b_;
    float x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = fmaf(x[i], a, b);
    float s = 0; for (int i = 0; i < ILP; ++i) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_imad(double* out, int iters, double a_, double b_) {
    uint32_t a = (uint32_t)(a_ * 1000) | 1u, b = (uint32_t)b_ + 7u;
    uint32_t x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = x[i] * a + b;
    uint32_t s = 0; for (int i = 0; i < ILP; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_iadd64(double* out, int iters, double a_, double b_) {
    uint64_t a = (uint64_t)(a_ * 1e12) | 1ull;
    uint64_t x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 0x9E3779B97F4A7C15ull + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = x[i] + (a ^ (uint64_t)i);
    uint64_t s = 0; for (int i = 0; i < ILP; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s >> 11) + b_;
}
__global__ void k_mul64hi(double* out, int iters, double a_, double b_) {
    uint64_t a = (uint64_t)(a_ * 1e15) | 1ull;
    uint64_t x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 0x9E3779B97F4A7C15ull + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = __umul64hi(x[i], a) + x[i];
    uint64_t s = 0; for (int i = 0; i < ILP; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s >> 11) + b_;
}
__global__ void k_smul64hi(double* out, int iters, double a_, double b_) {
    int64_t a = (int64_t)(a_ * 1e15) | 1ll;
    int64_t x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = (int64_t)(threadIdx.x * 0x9E3779B97F4A7C15ull + i);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = __mul64hi(x[i], a) + x[i];
    int64_t s = 0; for (int i = 0; i < ILP; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s >> 11) + b_;
}
__global__ void k_imadwide(double* out, int iters, double a_, double b_) {
    uint32_t a = (uint32_t)(a_ * 1000) | 1u;
    uint64_t x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] = (uint64_t)(uint32_t)x[i] * a + (x[i] >> 32);
    uint64_t s = 0; for (int i = 0; i < ILP; ++i) s ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)(s >> 11) + b_;
}
__global__ void k_copy(const double4_16a* __restrict__ in, double4_16a* __restrict__ out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) out[i] = in[i];
}



__global__ void k_i2d(double* out, int iters) {
    long long x[ILP]; double acc = 0;
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 977 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) { double d = (double)x[i]; x[i] = __double_as_longlong(d) >> 3; }
    for (int i = 0; i < ILP; ++i) acc += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}
__global__ void k_d2i(double* out, int iters) {
    double x[ILP]; long long acc = 0;
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 0.977 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) { long long v = __double2ll_rn(x[i]); x[i] = __longlong_as_double((v & 0xfffffffffffll) | 0x4000000000000000ll); }
    for (int i = 0; i < ILP; ++i) acc += __double_as_longlong(x[i]);
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)acc;
}
__global__ void k_dmul_conv(double* out, int iters, double w) {
    long long x[ILP];
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 977 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) x[i] += __double2ll_rn((double)x[i] * w);
    long long acc = 0; for (int i = 0; i < ILP; ++i) acc ^= x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = (double)acc;
}
__global__ void k_i2f32(double* out, int iters) {
    int x[ILP]; float acc = 0;
    for (int i = 0; i < ILP; ++i) x[i] = threadIdx.x * 977 + i;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int i = 0; i < ILP; ++i) { float f = (float)x[i]; x[i] = __float_as_int(f) >> 3; }
    for (int i = 0; i < ILP; ++i) acc += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}
template <class T, int Q, bool SHIFT>
__global__ void k_stream(const T* __restrict__ in, T* __restrict__ out, int nx, int ny, int nz) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= nx) return;
    const long long N = (long long)nx * ny * nz, c = ((long long)z * ny + y) * nx + x;
    const int sx[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
    const int sy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
    const int sz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
    const bool inner = x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1;
    T v[Q];
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        long long src = c;
        if (SHIFT && inner) src -= sx[n] + (long long)sy[n] * nx + (long long)sz[n] * nx * ny;
        v[n] = __ldg(in + n * N + src);
    }
#pragma unroll
    for (int n = 0; n < Q; ++n) out[n * N + c] = v[n] + (T)1;
}

typedef void (*kfn)(double*, int, double, double);


static int probes_pipes() {
    int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
    printf("device %s SMs %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
    const int blocks = p.multiProcessorCount * 8, threads = 256;
    double* out; CK(cudaMalloc(&out, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    struct { const char* name; kfn f; int iters; double ops_per_iter; } tests[] = {
        {"dfma (flop=2)", k_dfma, 2000, 2.0 * ILP},
        {"dadd", k_dadd, 2000, 1.0 * ILP},
        {"ddiv", k_ddiv, 200, 1.0 * ILP},
        {"ffma (flop=2)", k_ffma, 20000, 2.0 * ILP},
        {"imad32", k_imad, 20000, 1.0 * ILP},
        {"iadd64", k_iadd64, 20000, 1.0 * ILP},
        {"umul64hi+add", k_mul64hi, 5000, 1.0 * ILP},
        {"smul64hi+add", k_smul64hi, 5000, 1.0 * ILP},
        {"imad.wide32", k_imadwide, 10000, 1.0 * ILP},
    };
    for (auto& t : tests) {
        t.f<<<blocks, threads>>>(out, 10, 0.999, 1e-3);
        CK(cudaDeviceSynchronize());
        cudaEventRecord(e0);
        t.f<<<blocks, threads>>>(out, t.iters, 0.999, 1e-3);
        cudaEventRecord(e1);
        CK(cudaEventSynchronize(e1));
        float ms; cudaEventElapsedTime(&ms, e0, e1);
        double ops = (double)blocks * threads * t.iters * t.ops_per_iter;
        printf("%-16s %10.3f Gop/s  (%.3f ms)  per-SM-clk@1.9GHz %.2f\n", t.name, ops / ms / 1e6, ms,
               ops / (ms * 1e-3) / (p.multiProcessorCount * 1.9e9));
    }
    size_t n = (size_t)1 << 27;  // 128 Mi double4_16a = 4 GiB
    double4_16a *a, *b; CK(cudaMalloc(&a, n * sizeof(double4_16a))); CK(cudaMalloc(&b, n * sizeof(double4_16a)));
    CK(cudaMemset(a, 0, n * sizeof(double4_16a)));
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        k_copy<<<p.multiProcessorCount * 8, 512>>>(a, b, n);
        cudaEventRecord(e1);
        CK(cudaEventSynchronize(e1));
        float ms; cudaEventElapsedTime(&ms, e0, e1);
        printf("copy 4GiB: %.1f GB/s (r+w)\n", 2.0 * n * sizeof(double4_16a) / ms / 1e6);
    }
    cudaFree(a); cudaFree(b); cudaFree(out);
    return 0;
}


static int probes_conv_stream() {
    cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, 0));
    const int blocks = p.multiProcessorCount * 8, threads = 256;
    double* out; CK(cudaMalloc(&out, sizeof(double) * blocks * threads));
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    struct { const char* name; int iters; int which; } tests[] = {{"i2f.f64.s64 (+shift)", 2000, 0}, {"f2i.s64.f64 (+and/or)", 2000, 1},
                                                                  {"i2f64+dmul+f2i64+add", 1000, 2}, {"i2f.f32.s32 (+shift)", 20000, 3}};
    for (auto& t : tests) {
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(e0);
            if (t.which == 0) k_i2d<<<blocks, threads>>>(out, rep ? t.iters : 10);
            if (t.which == 1) k_d2i<<<blocks, threads>>>(out, rep ? t.iters : 10);
            if (t.which == 2) k_dmul_conv<<<blocks, threads>>>(out, rep ? t.iters : 10, 0.75);
            if (t.which == 3) k_i2f32<<<blocks, threads>>>(out, rep ? t.iters : 10);
            cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
            float ms; cudaEventElapsedTime(&ms, e0, e1);
            double ops = (double)blocks * threads * t.iters * ILP;
            if (rep) printf("%-24s %10.2f Gop/s  per-SM-clk@2.07GHz %.2f\n", t.name, ops / ms / 1e6, ops / (ms * 1e-3) / (p.multiProcessorCount * 2.07e9));
        }
    }
    // stream pattern at 512^3 for f32 and f64 (2 buffers each)
    const int n = 512;
    const long long N = (long long)n * n * n;
    for (int es = 4; es <= 8; es += 4) {
        void *a, *b;
        CK(cudaMalloc(&a, es * 19 * N)); CK(cudaMalloc(&b, es * 19 * N));
        CK(cudaMemset(a, 0, es * 19 * N));
        dim3 g(n / 256, n, n), blk(256);
        for (int sh = 0; sh < 2; ++sh) {
            float best = 1e9;
            for (int r = 0; r < 4; ++r) {
                cudaEventRecord(e0);
                if (es == 4) { if (sh) k_stream<float, 19, true><<<g, blk>>>((float*)a, (float*)b, n, n, n); else k_stream<float, 19, false><<<g, blk>>>((float*)a, (float*)b, n, n, n); }
                else { if (sh) k_stream<double, 19, true><<<g, blk>>>((double*)a, (double*)b, n, n, n); else k_stream<double, 19, false><<<g, blk>>>((double*)a, (double*)b, n, n, n); }
                cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
                float ms; cudaEventElapsedTime(&ms, e0, e1); if (ms < best) best = ms;
            }
            printf("stream19 %s %s: %.3f ms  %.1f GB/s  %.2f GLUPS\n", es == 4 ? "f32" : "f64", sh ? "pull-shift" : "aligned", best,
                   2.0 * es * 19 * N / best / 1e6, N / best / 1e6);
        }
        cudaFree(a); cudaFree(b);
    }
    return 0;
}

// Host link: page-locked host memory to the device and back, 4 GiB copies,
// one direction at a time and both at once on two streams (the bound of
// mph_step_host, which moves every population across the link twice).
static int probes_host_link() {
    const size_t bytes = (size_t)1 << 32;
    void *h0, *h1, *d0, *d1;
    CK(cudaHostAlloc(&h0, bytes, cudaHostAllocDefault));
    CK(cudaHostAlloc(&h1, bytes, cudaHostAllocDefault));
    CK(cudaMalloc(&d0, bytes));
    CK(cudaMalloc(&d1, bytes));
    CK(cudaMemset(d1, 0, bytes));
    for (size_t i = 0; i < bytes; i += 4096) static_cast<char*>(h0)[i] = 1;  // touch the pages
    cudaStream_t s0, s1;
    CK(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    for (int mode = 0; mode < 3; ++mode) {  // h2d, d2h, both
        float best = 1e9;
        for (int r = 0; r < 3; ++r) {
            CK(cudaDeviceSynchronize());
            cudaEventRecord(e0, s0);
            CK(cudaStreamWaitEvent(s1, e0, 0));
            if (mode != 1) CK(cudaMemcpyAsync(d0, h0, bytes, cudaMemcpyHostToDevice, s0));
            if (mode != 0) CK(cudaMemcpyAsync(h1, d1, bytes, cudaMemcpyDeviceToHost, mode == 2 ? s1 : s0));
            cudaEvent_t done; cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
            cudaEventRecord(done, s1);
            CK(cudaStreamWaitEvent(s0, done, 0));
            cudaEventRecord(e1, s0);
            CK(cudaEventSynchronize(e1));
            cudaEventDestroy(done);
            float ms; cudaEventElapsedTime(&ms, e0, e1); if (ms < best) best = ms;
        }
        const double moved = (mode == 2 ? 2.0 : 1.0) * (double)bytes;
        printf("host link %s: %.1f GB/s\n", mode == 0 ? "host->device" : mode == 1 ? "device->host" : "both at once", moved / best / 1e6);
    }
    cudaStreamDestroy(s0); cudaStreamDestroy(s1);
    cudaFreeHost(h0); cudaFreeHost(h1); cudaFree(d0); cudaFree(d1);
    return 0;
}

int main() { return probes_pipes() | probes_conv_stream() | probes_host_link(); }
