// noalloc.cu -- FP64 population sums (mass and momentum) for callers that
// cannot allocate device memory.
//
// mph_reduce keeps its block partials in scratch that the simulation handle
// allocates with cudaMalloc.  Some callers of the step cannot do that: a
// solver embedded in an application whose memory arena already holds nearly
// all device memory (AMReX reserves a large arena at start-up, so a separate
// cudaMalloc can fail), or a caller with a no-allocation-after-start-up
// policy, where cudaMalloc's implicit device synchronisation would also stall
// its asynchronous pipeline.  mph_reduce_f64_noalloc works on caller-owned
// populations and output and keeps its partials in the fixed array below,
// which is part of the loaded library image on every device that uses it.
#include <mutex>
#include <string>

#include "lattice.cuh"
#include "mph_internal.h"

namespace {

// Each block reduces one contiguous chunk of kChunkCells cells; kSlots chunk
// slots bound the problem size at kSlots * kChunkCells = 134,217,728 cells
// (a 512^3 grid).  4 partials per slot: 64 KiB of device memory.
constexpr int kSlots = 2048;
constexpr long long kChunkCells = 65536;
constexpr long long kMaxCells = kSlots * kChunkCells;

static __device__ __align__(256) double g_partials[4 * kSlots];

// Device address of g_partials, looked up once per device.  The host-side
// name g_partials is only a stand-in for the symbol, not a device address.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

int scratch_address(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return mph::fail(MPH_ERR_ARG, "mph_reduce_f64_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess)
            return mph::fail(MPH_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return MPH_OK;
}

template <int Q>
__global__ void __launch_bounds__(256) k_chunk_sums(const double* __restrict__ f, long long ncell,
                                                    double* __restrict__ part) {
    using L = mph::Lat<Q>;
    const long long c0 = (long long)blockIdx.x * kChunkCells;
    const long long c1 = (c0 + kChunkCells < ncell) ? c0 + kChunkCells : ncell;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
#pragma unroll
        for (int n = 0; n < Q; ++n) {
            const double v = __ldg(f + n * ncell + c);
            a[0] += v;
            if (L::cx(n)) a[1] += L::cx(n) * v;
            if (L::cy(n)) a[2] += L::cy(n) * v;
            if (L::cz(n)) a[3] += L::cz(n) * v;
        }
    }
    __shared__ double sh[4][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double v = a[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) sh[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
        part[4 * blockIdx.x + threadIdx.x] = v;
    }
}

// Adds the partials of slots 0..nblocks-1, all written by k_chunk_sums of the
// same call, in a fixed order.
__global__ void k_sum_slots(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 4) return;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += part[4 * b + k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) out[k] = v;
}

}  // namespace

extern "C" int mph_reduce_f64_noalloc(int dim, int q, const double* f, long long ncell, double* out, void* stream) {
    if (!mph::lattice_ok(dim, q)) return mph::fail(MPH_ERR_ARG, "mph_reduce_f64_noalloc: unsupported lattice (dim, q)");
    if (!f || !out) return mph::fail(MPH_ERR_ARG, "mph_reduce_f64_noalloc: NULL pointer");
    if (ncell < 1) return mph::fail(MPH_ERR_ARG, "mph_reduce_f64_noalloc: ncell must be positive");
    if (ncell > kMaxCells)
        return mph::fail(MPH_ERR_ARG, "mph_reduce_f64_noalloc: " + std::to_string(ncell) +
                                          " cells exceed the fixed scratch capacity of " + std::to_string(kMaxCells) +
                                          " cells (2048 slots x 65536 cells)");
    double* part = nullptr;
    int rc = scratch_address(&part);
    if (rc) return rc;
    const int nblocks = (int)((ncell + kChunkCells - 1) / kChunkCells);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (q) {
        case 9: k_chunk_sums<9><<<nblocks, 256, 0, s>>>(f, ncell, part); break;
        case 15: k_chunk_sums<15><<<nblocks, 256, 0, s>>>(f, ncell, part); break;
        case 19: k_chunk_sums<19><<<nblocks, 256, 0, s>>>(f, ncell, part); break;
        case 27: k_chunk_sums<27><<<nblocks, 256, 0, s>>>(f, ncell, part); break;
    }
    k_sum_slots<<<1, 128, 0, s>>>(part, nblocks, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return mph::fail(MPH_ERR_CUDA, std::string("mph_reduce_f64_noalloc launch: ") + cudaGetErrorString(e));
    return MPH_OK;
}
