// nn.cu -- kernels of the warm-start surrogate (no counterpart in the
// reference): a small convolutional U-Net over NHWC activations, trained and
// evaluated on the GPU with these kernels only.
//
//   * gemm_bf16: C (FP32) [+]= A . B with BF16 operands on the tensor cores
//     (mma.sync m16n8k16, FP32 accumulation), 64 x 64 x 32 block tiles staged
//     through shared memory; either operand may be stored transposed, so the
//     forward pass (X_col . W), the data gradient (dY . W^T) and the weight
//     gradient (X_col^T . dY) of a 3 x 3 convolution are the same kernel.
//   * im2col / col2im for 3 x 3, pad 1 convolutions (col2im gathers, so the
//     data gradient is deterministic), bias + leaky ReLU (forward, backward,
//     bias gradient), 2 x 2 average pooling, nearest 2x upsampling, channel
//     concatenation, masked MSE loss, Adam on FP32 master weights, casts, and
//     device buffers for a host driver without its own allocator.
//
// Shapes: activations [P][C] with P = batch x H x W pixels (NHWC), weights of
// a 3 x 3 conv as Wt [Cout][9 Cin] (k = (dy * 3 + dx) * Cin + ci contiguous).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "mph.h"
#include "mph_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int BM = 64, BN = 64, BK = 32, KPAD = 8;


__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[m][n] (ldc) = sum_k A(m, k) B(k, n) (+ C if accumulate).
// A(m, k) = TA ? A[k * lda + m] : A[m * lda + k]
// B(k, n) = TB ? B[k * ldb + n] : B[n * ldb + k]
// 128 threads: warp w computes rows (w / 2) * 32 .. +32, cols (w % 2) * 32 .. +32.
// Split K: blockIdx.z covers k in [z kchunk, (z + 1) kchunk) and, with more
// than one split, writes its partial product to C + z M ldc (a workspace that
// k_splitk_reduce adds up in split order).
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const bf16* __restrict__ A, long long lda,
                                                   const bf16* __restrict__ B, long long ldb, float* __restrict__ C,
                                                   long long ldc, int accumulate, int kchunk) {
    __shared__ __align__(16) bf16 As[BM][BK + KPAD];
    __shared__ __align__(16) bf16 Bs[BN][BK + KPAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const long long m0 = (long long)blockIdx.y * BM, n0 = (long long)blockIdx.x * BN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
    const bf16 zero = __float2bfloat16(0.f);
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    C += (long long)blockIdx.z * M * ldc;
    for (int k0 = kb; k0 < ke; k0 += BK) {
        // Stage A and B tiles (64 x 32 each: 2048 values, 16 per thread).
#pragma unroll 4
        for (int e = tid; e < BM * BK; e += 128) {
            int r, c;
            if (TA) { c = e / BM; r = e % BM; } else { r = e / BK; c = e % BK; }
            const long long gm = m0 + r;
            const int gk = k0 + c;
            bf16 v = zero;
            if (gm < M && gk < ke) v = TA ? A[(long long)gk * lda + gm] : A[gm * lda + gk];
            As[r][c] = v;
        }
#pragma unroll 4
        for (int e = tid; e < BN * BK; e += 128) {
            int r, c;
            if (TB) { c = e / BN; r = e % BN; } else { r = e / BK; c = e % BK; }
            const long long gn = n0 + r;
            const int gk = k0 + c;
            bf16 v = zero;
            if (gn < N && gk < ke) v = TB ? B[(long long)gk * ldb + gn] : B[gn * ldb + gk];
            Bs[r][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            unsigned af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + g;
                af[i][0] = *reinterpret_cast<const unsigned*>(&As[r][kk + 2 * t]);
                af[i][1] = *reinterpret_cast<const unsigned*>(&As[r + 8][kk + 2 * t]);
                af[i][2] = *reinterpret_cast<const unsigned*>(&As[r][kk + 2 * t + 8]);
                af[i][3] = *reinterpret_cast<const unsigned*>(&As[r + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int cidx = wn + j * 8 + g;
                bfr[j][0] = *reinterpret_cast<const unsigned*>(&Bs[cidx][kk + 2 * t]);
                bfr[j][1] = *reinterpret_cast<const unsigned*>(&Bs[cidx][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const long long row = m0 + wm + i * 16 + g + (r >= 2 ? 8 : 0);
                const long long col = n0 + wn + j * 8 + 2 * t + (r & 1);
                if (row < M && col < N) {
                    float* p = C + row * ldc + col;
                    *p = accumulate ? *p + acc[i][j][r] : acc[i][j][r];
                }
            }
}

// ---- tcgen05 GEMM (5th-generation tensor cores, accumulator in TMEM) ------
// Same contract as k_gemm_bf16.  One CTA of 128 threads computes a 128 x 64
// tile of C: per 64-wide K step all threads stage A (128 x 64) and B (64 x 64)
// into shared memory in the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per 128-byte core matrix, core matrices contiguous along K, 1 KiB
// apart along M / N), one thread issues four tcgen05.mma (M 128, N 64, K 16,
// BF16 in, FP32 accumulate in TMEM) and commits them to an mbarrier that every
// thread waits on before the buffer is refilled.  Each warp then reads its 32
// TMEM lanes (rows) with tcgen05.ld.  Every wait is bounded: on timeout the
// kernel records an error flag and skips its tile.  The outcome of a wait is
// combined over the block (__syncthreads_and) before anything depends on it,
// so every thread leaves the K loop at the same iteration and the warp-
// collective tcgen05.ld / dealloc see one decision.  After a timeout the
// dealloc is best effort: MMAs still in flight may write the released
// columns, and the tile's result is discarded.
constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 64;
// A wait gives up after kWaitNs of %globaltimer time (checked every 256
// polls) or kSpinLimit polls, whichever comes first.
constexpr unsigned long long kSpinLimit = 1ull << 26;
constexpr unsigned long long kWaitNs = 250ull * 1000 * 1000;

__device__ int g_nn_timeout = 0;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Bounded wait for phase `phase` of the mbarrier at shared address `addr`.
__device__ __forceinline__ bool mbar_wait(unsigned addr, unsigned phase) {
    unsigned done = 0;
    const unsigned long long t0 = global_ns();
    for (unsigned long long it = 0; it < kSpinLimit && !done; ++it) {
        asm volatile(
            "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\nselp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase));
        if (!done && (it & 255) == 255 && global_ns() - t0 > kWaitNs) break;
    }
    return done != 0;
}

// Core-matrix layout offset (bytes) of element (row, k) in a rows x TC_BK tile.
__device__ __forceinline__ unsigned cm_off(int row, int k) {
    return (unsigned)((((row >> 3) * (TC_BK / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ unsigned long long smem_desc(unsigned addr) {
    const unsigned long long lbo = 128 >> 4, sbo = ((TC_BK / 8) * 128) >> 4;
    return (unsigned long long)((addr >> 4) & 0x3FFF) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_tc05(int M, int N, int K, const bf16* __restrict__ A, long long lda,
                                                   const bf16* __restrict__ B, long long ldb, float* __restrict__ C,
                                                   long long ldc, int accumulate, int kchunk) {
    __shared__ __align__(1024) unsigned char As[TC_BM * TC_BK * 2];
    __shared__ __align__(1024) unsigned char Bs[TC_BN * TC_BK * 2];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ unsigned tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long m0 = (long long)blockIdx.y * TC_BM, n0 = (long long)blockIdx.x * TC_BN;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = tmem_base;
    const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(TC_BN >> 3) << 17) |
                           ((unsigned)(TC_BM >> 4) << 24);
    const bf16 zero = __float2bfloat16(0.f);
    // 16-byte loads need 16-byte aligned bases (element offsets are checked per chunk)
    const bool a_vec = (reinterpret_cast<unsigned long long>(A) & 15) == 0;
    const bool b_vec = (reinterpret_cast<unsigned long long>(B) & 15) == 0;
    unsigned phase = 0;
    bool ok = true;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    C += (long long)blockIdx.z * M * ldc;
    for (int k0 = kb; k0 < ke && ok; k0 += TC_BK) {
        // A: 128 rows x 8 chunks of 8 k-values; thread handles chunks tid + 128 i.
#pragma unroll 2
        for (int ch = tid; ch < TC_BM * (TC_BK / 8); ch += 128) {
            const int row = ch % TC_BM, kc = ch / TC_BM;
            const long long gm = m0 + row;
            const int gk0 = k0 + kc * 8;
            if (!TA && a_vec && gm < M && gk0 + 8 <= ke && ((gm * lda + gk0) & 7) == 0) {
                // eight K-contiguous values: one 16-byte load
                *reinterpret_cast<uint4*>(As + cm_off(row, kc * 8)) = __ldg(reinterpret_cast<const uint4*>(A + gm * lda + gk0));
                continue;
            }
            unsigned short v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int gk = gk0 + j;
                bf16 x = zero;
                if (gm < M && gk < ke) x = TA ? A[(long long)gk * lda + gm] : A[gm * lda + gk];
                v[j] = __bfloat16_as_ushort(x);
            }
            uint4 w;
            w.x = v[0] | ((unsigned)v[1] << 16);
            w.y = v[2] | ((unsigned)v[3] << 16);
            w.z = v[4] | ((unsigned)v[5] << 16);
            w.w = v[6] | ((unsigned)v[7] << 16);
            *reinterpret_cast<uint4*>(As + cm_off(row, kc * 8)) = w;
        }
#pragma unroll 2
        for (int ch = tid; ch < TC_BN * (TC_BK / 8); ch += 128) {
            const int row = ch % TC_BN, kc = ch / TC_BN;
            const long long gn = n0 + row;
            const int gk0 = k0 + kc * 8;
            if (!TB && b_vec && gn < N && gk0 + 8 <= ke && ((gn * ldb + gk0) & 7) == 0) {
                *reinterpret_cast<uint4*>(Bs + cm_off(row, kc * 8)) = __ldg(reinterpret_cast<const uint4*>(B + gn * ldb + gk0));
                continue;
            }
            unsigned short v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int gk = gk0 + j;
                bf16 x = zero;
                if (gn < N && gk < ke) x = TB ? B[(long long)gk * ldb + gn] : B[gn * ldb + gk];
                v[j] = __bfloat16_as_ushort(x);
            }
            uint4 w;
            w.x = v[0] | ((unsigned)v[1] << 16);
            w.y = v[2] | ((unsigned)v[3] << 16);
            w.z = v[4] | ((unsigned)v[5] << 16);
            w.w = v[6] | ((unsigned)v[7] << 16);
            *reinterpret_cast<uint4*>(Bs + cm_off(row, kc * 8)) = w;
        }
        // Generic-proxy stores must be visible to the tensor core's async proxy.
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk) {
                // K step of 16 = two core matrices = 256 bytes
                const unsigned long long ad = smem_desc(smem_u32(As) + kk * 256);
                const unsigned long long bd = smem_desc(smem_u32(Bs) + kk * 256);
                const unsigned acc = (k0 > kb || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&mbar)));
        }
        // Every thread waits for the MMAs (they read the staged tiles); the
        // block continues only if every thread's wait succeeded.
        const bool done = mbar_wait(smem_u32(&mbar), phase);
        phase ^= 1;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        ok = __syncthreads_and(done) != 0;
        if (!ok && tid == 0) atomicExch(&g_nn_timeout, 1);
    }
    if (ok) {
        // Warp w reads TMEM lanes 32 w .. 32 w + 31 (rows), 64 columns.
        float acc[TC_BN];
        unsigned r[TC_BN];
        const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
            "%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,"
            "%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
              "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
              "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
              "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
              "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int j = 0; j < TC_BN; ++j) acc[j] = __uint_as_float(r[j]);
        const long long row = m0 + 32 * warp + lane;
        if (row < M) {
            float* crow = C + row * ldc + n0;
#pragma unroll
            for (int j = 0; j < TC_BN; ++j)
                if (n0 + j < N) crow[j] = accumulate ? crow[j] + acc[j] : acc[j];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_BN));
}

// Pipelined variant: three shared-memory stages of 32-wide K slices.  Rows
// that are K-contiguous and 16-byte aligned arrive by cp.async (16 bytes per
// core-matrix row), others by plain loads; while the tensor core works on
// slice t the threads fill slice t + 2.  Each stage's mbarrier is waited on
// (bounded) before the stage is refilled, and the last commit before the
// accumulator is read.
constexpr int TP_BK = 32, TP_STAGES = 3;
constexpr int TP_A_BYTES = TC_BM * TP_BK * 2, TP_B_BYTES = TC_BN * TP_BK * 2;

__device__ __forceinline__ unsigned cm_off32(int row, int k) {
    return (unsigned)((((row >> 3) * (TP_BK / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ unsigned long long smem_desc32(unsigned addr) {
    const unsigned long long lbo = 128 >> 4, sbo = ((TP_BK / 8) * 128) >> 4;
    return (unsigned long long)((addr >> 4) & 0x3FFF) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// One rows x 32 K slice of an operand into stage memory `dst`.
template <bool T, int ROWS>
__device__ __forceinline__ void tp_stage(unsigned char* dst, const bf16* __restrict__ X, long long ld, long long r0,
                                         long long rmax, int k0, int ke, bool vec_ok) {
    const bf16 zero = __float2bfloat16(0.f);
    for (int ch = threadIdx.x; ch < ROWS * (TP_BK / 8); ch += 128) {
        const int row = ch % ROWS, kc = ch / ROWS;
        const long long gr = r0 + row;
        const int gk0 = k0 + kc * 8;
        unsigned char* d = dst + cm_off32(row, kc * 8);
        if (!T && vec_ok && gr < rmax && gk0 + 8 <= ke && ((gr * ld + gk0) & 7) == 0) {
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(d)), "l"(X + gr * ld + gk0)
                         : "memory");
            continue;
        }
        unsigned short v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gk = gk0 + j;
            bf16 x = zero;
            if (gr < rmax && gk < ke) x = T ? X[(long long)gk * ld + gr] : X[gr * ld + gk];
            v[j] = __bfloat16_as_ushort(x);
        }
        uint4 w;
        w.x = v[0] | ((unsigned)v[1] << 16);
        w.y = v[2] | ((unsigned)v[3] << 16);
        w.z = v[4] | ((unsigned)v[5] << 16);
        w.w = v[6] | ((unsigned)v[7] << 16);
        *reinterpret_cast<uint4*>(d) = w;
    }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_tc05p(int M, int N, int K, const bf16* __restrict__ A, long long lda,
                                                    const bf16* __restrict__ B, long long ldb, float* __restrict__ C,
                                                    long long ldc, int accumulate, int kchunk) {
    __shared__ __align__(1024) unsigned char As[TP_STAGES][TP_A_BYTES];
    __shared__ __align__(1024) unsigned char Bs[TP_STAGES][TP_B_BYTES];
    __shared__ __align__(8) unsigned long long mbar[TP_STAGES];
    __shared__ unsigned tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long m0 = (long long)blockIdx.y * TC_BM, n0 = (long long)blockIdx.x * TC_BN;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int s = 0; s < TP_STAGES; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[s])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = tmem_base;
    const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(TC_BN >> 3) << 17) |
                           ((unsigned)(TC_BM >> 4) << 24);
    const bool a_vec = (reinterpret_cast<unsigned long long>(A) & 15) == 0;
    const bool b_vec = (reinterpret_cast<unsigned long long>(B) & 15) == 0;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    const int nk = (ke - kb + TP_BK - 1) / TP_BK;
    C += (long long)blockIdx.z * M * ldc;
    unsigned phase[TP_STAGES] = {0, 0, 0};
    bool ok = true;
    // prologue: slices 0 .. STAGES-2
    for (int s = 0; s < TP_STAGES - 1; ++s) {
        if (s < nk) {
            tp_stage<TA, TC_BM>(As[s], A, lda, m0, M, kb + s * TP_BK, ke, a_vec);
            tp_stage<TB, TC_BN>(Bs[s], B, ldb, n0, N, kb + s * TP_BK, ke, b_vec);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    for (int t = 0; t < nk && ok; ++t) {
        const int s = t % TP_STAGES;
        asm volatile("cp.async.wait_group %0;\n" ::"n"(TP_STAGES - 2) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < TP_BK / 16; ++kk) {
                const unsigned long long ad = smem_desc32(smem_u32(As[s]) + kk * 256);
                const unsigned long long bd = smem_desc32(smem_u32(Bs[s]) + kk * 256);
                const unsigned acc = (t > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&mbar[s])));
        }
        // refill the stage of slice t - 1 with slice t + STAGES - 1
        const int tn = t + TP_STAGES - 1;
        if (tn < nk) {  // uniform over the block (t and nk are)
            const int sn = tn % TP_STAGES;
            if (t >= 1) {
                const bool done = mbar_wait(smem_u32(&mbar[sn]), phase[sn]);
                phase[sn] ^= 1;
                ok = __syncthreads_and(done) != 0;
                if (!ok && tid == 0) atomicExch(&g_nn_timeout, 1);
            }
            if (ok) {
                tp_stage<TA, TC_BM>(As[sn], A, lda, m0, M, kb + tn * TP_BK, ke, a_vec);
                tp_stage<TB, TC_BN>(Bs[sn], B, ldb, n0, N, kb + tn * TP_BK, ke, b_vec);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    bool done = true;
    if (ok) done = mbar_wait(smem_u32(&mbar[(nk - 1) % TP_STAGES]), phase[(nk - 1) % TP_STAGES]);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const bool last_ok = __syncthreads_and(done) != 0;
    if (ok && !last_ok && tid == 0) atomicExch(&g_nn_timeout, 1);
    ok = ok && last_ok;
    if (ok) {
        float acc[TC_BN];
        unsigned r[TC_BN];
        const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
            "%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,"
            "%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
              "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
              "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
              "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
              "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
        for (int j = 0; j < TC_BN; ++j) acc[j] = __uint_as_float(r[j]);
        const long long row = m0 + 32 * warp + lane;
        if (row < M) {
            float* crow = C + row * ldc + n0;
#pragma unroll
            for (int j = 0; j < TC_BN; ++j)
                if (n0 + j < N) crow[j] = accumulate ? crow[j] + acc[j] : acc[j];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_BN));
}

// ---- TMA-fed tcgen05 GEMM (both operands K-contiguous) --------------------
// Same contract as k_gemm_tc05p for ta = tb = 0.  A 128 x BN tile of C per CTA
// of 128 threads; K in slices of 64 through a ring of TM_STAGES stages:
//   thread 0 (producer): waits for the stage to be empty, announces the bytes
//     on its `full` mbarrier and issues two tiled TMA copies
//     (cp.async.bulk.tensor.2d, 128-byte swizzle: the A slice is 128 rows x
//     128 B, the B slice BN rows x 128 B; rows / columns past M, N or K read as
//     zeros);
//   thread 32 (MMA issuer): waits for the stage to be full and issues four
//     tcgen05.mma (M 128, N BN, K 16) on 128-byte-swizzled K-major shared-memory
//     descriptors (8-row atoms 1024 B apart, the K step advances the start
//     address by 32 B inside the atom), then tcgen05.commit to the stage's
//     `empty` mbarrier, and after the last slice to `done`;
//   all warps: wait for `done`, read the FP32 accumulator from TMEM in 32-column
//     pieces (tcgen05.ld.32x32b.x32), transpose it through shared memory (the
//     stage buffers, free by then) and write C rows with consecutive lanes on
//     consecutive columns.
// Every wait is bounded (mbar_wait); the outcome is combined over the block
// before the warp-collective TMEM reads, and a timeout sets g_nn_timeout.
//
// Template parameters: BKC = K elements per slice, 64 (128-byte rows, 128-byte
// swizzle) or 32 (64-byte rows, 64-byte swizzle, for 32-channel convolutions);
// CONV = implicit-GEMM 3 x 3 convolution: A is not a matrix in memory but the
// NHWC activation X [B][H][W][C] seen through a 4-D tensor map (C, W, H, B);
// the 128 rows of an M tile are 128 consecutive pixels (whole image rows, or
// a 128-pixel piece of one), and the A slice of K index k = t C + c0 (tap t =
// 3 dy + dx) is the box of BKC channels at (c0, x0 + dx - 1, y0 + dy - 1, b):
// the tap's shifted pixels, with the padding read as zeros by TMA (coordinates
// outside the image).  So A(p, t C + c) = X[pixel p shifted by tap t][c], the
// im2col matrix, without writing it.
constexpr int TM_STAGES = 4;

struct ConvGeom {
    int C, H, W;  // channels, height, width of the activation (CONV kernels)
};

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// K-major shared-memory matrix descriptor of a swizzled tile: rows of BKC * 2
// bytes, atoms of 8 rows (stride byte offset 8 rows), leading byte offset
// unused (1), descriptor version 1 (bits 46-47), layout type at bits 61-63:
// 2 = 128-byte swizzle (BKC 64), 4 = 64-byte swizzle (BKC 32).
template <int BKC>
__device__ __forceinline__ unsigned long long smem_desc_sw(unsigned addr) {
    constexpr unsigned long long sbo = (8 * BKC * 2) >> 4, layout = BKC == 64 ? 2ull : 4ull;
    return (unsigned long long)((addr >> 4) & 0x3FFF) | (1ull << 16) | (sbo << 32) | (1ull << 46) | (layout << 61);
}

template <int BN, int BKC, bool CONV>
__global__ void __launch_bounds__(128) k_gemm_tma(int M, int N, const __grid_constant__ CUtensorMap tmA,
                                                  const __grid_constant__ CUtensorMap tmB, float* __restrict__ C,
                                                  long long ldc, int accumulate, int K, int kchunk, const ConvGeom cg) {
    constexpr int TM_BK = BKC;
    constexpr int A_BYTES = 128 * TM_BK * 2, B_BYTES = BN * TM_BK * 2;
    extern __shared__ unsigned char tm_dyn[];
    __shared__ __align__(8) unsigned long long full[TM_STAGES], empty[TM_STAGES], done;
    __shared__ unsigned tmem_base;
    // stage buffers on a 1024-byte boundary (the swizzle atom)
    unsigned char* base = tm_dyn + ((1024u - (smem_u32(tm_dyn) & 1023u)) & 1023u);
    unsigned char* sA = base;
    unsigned char* sB = base + TM_STAGES * A_BYTES;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    const int nk = (ke - kb + TM_BK - 1) / TM_BK;
    C += (long long)blockIdx.z * M * ldc;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int s = 0; s < TM_STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<unsigned long long>(&tmB)) : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    const unsigned tmem = tmem_base;
    bool ok = true;
    if (tid == 0) {  // producer
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % TM_STAGES, u = kt / TM_STAGES;
            if (u > 0 && !mbar_wait(smem_u32(&empty[s]), (unsigned)(u - 1) & 1u)) {
                ok = false;
                break;
            }
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(&full[s])),
                         "r"(A_BYTES + B_BYTES)
                         : "memory");
            const int k = kb + kt * TM_BK;
            if constexpr (CONV) {
                // M tile -> first pixel (b, y0, x0); K index -> tap and channel block
                const int hw = cg.H * cg.W;
                const int b = m0 / hw, rem = m0 - b * hw;
                const int y0 = rem / cg.W, x0 = rem - y0 * cg.W;
                const int t = k / cg.C, c0 = k - t * cg.C;
                const int dy = t / 3, dx = t - 3 * dy;
                tma_load_4d(sA + s * A_BYTES, &tmA, c0, x0 + dx - 1, y0 + dy - 1, b, &full[s]);
            } else {
                tma_load_2d(sA + s * A_BYTES, &tmA, k, m0, &full[s]);
            }
            tma_load_2d(sB + s * B_BYTES, &tmB, k, n0, &full[s]);
        }
    } else if (tid == 32) {  // MMA issuer
        const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(BN >> 3) << 17) | ((unsigned)(128 >> 4) << 24);
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % TM_STAGES, u = kt / TM_STAGES;
            if (!mbar_wait(smem_u32(&full[s]), (unsigned)u & 1u)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
#pragma unroll
            for (int kk = 0; kk < TM_BK / 16; ++kk) {
                const unsigned long long ad = smem_desc_sw<BKC>(smem_u32(sA + s * A_BYTES) + kk * 32);
                const unsigned long long bd = smem_desc_sw<BKC>(smem_u32(sB + s * B_BYTES) + kk * 32);
                const unsigned acc = (kt > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&empty[s])));
        }
        if (ok)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                smem_u32(&done)));
    }
    __syncwarp();
    const bool got = ok && mbar_wait(smem_u32(&done), 0u);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    ok = __syncthreads_and(got) != 0;
    if (!ok && tid == 0) atomicExch(&g_nn_timeout, 1);
    if (ok) {
        // TMEM -> registers -> shared memory tile [128][BN + 1] -> coalesced rows of C
        float* tile = reinterpret_cast<float*>(base);
        constexpr int LD = BN + 1;
        const int row = 32 * warp + lane;
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 32) {
            unsigned r[32];
            const unsigned taddr = tmem + ((unsigned)(32 * warp) << 16) + (unsigned)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
                "%28,%29,%30,%31}, [%32];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                  "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; ++j) tile[row * LD + c0 + j] = __uint_as_float(r[j]);
        }
        __syncwarp();
        for (int rr = 0; rr < 32; ++rr) {
            const int trow = 32 * warp + rr;
            const int gm = m0 + trow;
            if (gm >= M) break;
            float* crow = C + (long long)gm * ldc + n0;
            for (int c = lane; c < BN; c += 32)
                if (n0 + c < N) crow[c] = accumulate ? crow[c] + tile[trow * LD + c] : tile[trow * LD + c];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

// Stage memory, also holding the 128 x (BN + 1) FP32 epilogue tile.
template <int BN, int BKC>
constexpr size_t tma_smem_bytes() {
    constexpr size_t stages = (size_t)TM_STAGES * (128 + BN) * BKC * 2, tile = (size_t)128 * (BN + 1) * 4;
    return 1024 + (stages > tile ? stages : tile);
}

// C[m][n] (+)= sum over splits z of W[z][m][n] (W rows of width N), in split order.
// C[m][n] (+)= sum over splits z of W[z][m][n], in split order (few splits).
__global__ void k_splitk_reduce(const float* __restrict__ W, int S, int M, int N, float* __restrict__ C, long long ldc,
                                int accumulate) {
    const long long total = (long long)M * N;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < S; ++z) s += W[(long long)z * total + i];
        const long long m = i / N, n = i % N;
        float* p = C + m * ldc + n;
        *p = accumulate ? *p + s : s;
    }
}

// Many splits (the weight gradients, K = pixels): blocks of 256 threads, 64
// elements x 4 groups of consecutive splits; each group adds its splits in
// order, then the four group sums are added in group order (a fixed order:
// the result is the same on every call).
__global__ void __launch_bounds__(256) k_splitk_reduce4(const float* __restrict__ W, int S, int M, int N,
                                                       float* __restrict__ C, long long ldc, int accumulate) {
    __shared__ float part[4][64];
    const long long total = (long long)M * N;
    const int e = threadIdx.x & 63, grp = threadIdx.x >> 6;
    const long long i = (long long)blockIdx.x * 64 + e;
    const int per = (S + 3) / 4, z0 = grp * per, z1 = min(S, z0 + per);
    float t = 0.f;
    if (i < total)
        for (int z = z0; z < z1; ++z) t += W[(long long)z * total + i];
    part[grp][e] = t;
    __syncthreads();
    if (grp == 0 && i < total) {
        const float sum = ((part[0][e] + part[1][e]) + part[2][e]) + part[3][e];
        const long long m = i / N, n = i - m * N;
        float* p = C + m * ldc + n;
        *p = accumulate ? *p + sum : sum;
    }
}

// ---- convolution data movement --------------------------------------------
// im2col with 16-byte moves (C a multiple of 8, 32-bit index math): one
// thread per (pixel, tap, 8-channel group); consecutive threads read and
// write consecutive 16-byte groups.
__global__ void __launch_bounds__(256) k_im2col3_v8(const uint4* __restrict__ X, int Bn, int H, int W, int G,
                                                    uint4* __restrict__ Xcol) {
    const unsigned total = (unsigned)Bn * H * W * 9u * G;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const unsigned g = i % G, r = i / G;
    const unsigned tap = r % 9u, p = r / 9u;
    const unsigned x = p % W, q = p / W;
    const unsigned y = q % H, b = q / H;
    const int sy = (int)y + (int)(tap / 3u) - 1, sx = (int)x + (int)(tap % 3u) - 1;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (sy >= 0 && sy < H && sx >= 0 && sx < W) v = X[((b * H + sy) * (unsigned)W + sx) * G + g];
    Xcol[i] = v;
}

// Xcol[p][(dy * 3 + dx) * C + c] = X[b][y + dy - 1][x + dx - 1][c] (0 outside).
__global__ void k_im2col3(const bf16* __restrict__ X, int Bn, int H, int W, int C, bf16* __restrict__ Xcol) {
    const long long total = (long long)Bn * H * W * 9 * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long r = i / C;
        const int tap = (int)(r % 9);
        const long long p = r / 9;
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        const int sy = y + tap / 3 - 1, sx = x + tap % 3 - 1;
        bf16 v = __float2bfloat16(0.f);
        if (sy >= 0 && sy < H && sx >= 0 && sx < W) v = X[((b * H + sy) * W + sx) * C + c];
        Xcol[i] = v;
    }
}

// dX[b][y][x][c] = sum over taps of dXcol at the pixel that read (y, x).
__global__ void k_col2im3(const float* __restrict__ dXcol, int Bn, int H, int W, int C, float* __restrict__ dX) {
    const long long total = (long long)Bn * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        float s = 0.f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int oy = y - (tap / 3 - 1), ox = x - (tap % 3 - 1);  // output pixel whose tap read (y, x)
            if (oy >= 0 && oy < H && ox >= 0 && ox < W)
                s += dXcol[(((b * H + oy) * W + ox) * 9 + tap) * (long long)C + c];
        }
        dX[i] = s;
    }
}

// out[p][c] = leaky(Y[p][c] + bias[c]) as BF16 into a channel slice of width
// ld_out starting at column c_off; leaky slope 0.1 (act = 1), identity (0).
__global__ void k_bias_act(const float* __restrict__ Y, const float* __restrict__ bias, long long P, int C, int act,
                           bf16* __restrict__ out_bf, float* __restrict__ out_f, int ld_out, int c_off) {
    const long long total = P * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        // 32-bit division while the index fits (a 64-bit one costs several times more)
        const bool small = total < (1LL << 32);
        const int c = small ? (int)((unsigned)i % (unsigned)C) : (int)(i % C);
        const long long p = small ? (long long)((unsigned)i / (unsigned)C) : i / C;
        float v = Y[i] + bias[c];
        if (act && v < 0.f) v *= 0.1f;
        if (out_bf) out_bf[p * ld_out + c_off + c] = __float2bfloat16(v);
        if (out_f) out_f[p * ld_out + c_off + c] = v;
    }
}

// dPre = dOut * leaky'(pre), reading the sign from the stored activation.
__global__ void k_act_bwd(const float* __restrict__ dOut, int ld_dout, int c_off, const bf16* __restrict__ act_out,
                          int ld_act, int act_off, long long P, int C, int act, float* __restrict__ dPre) {
    const long long total = P * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const bool small = total < (1LL << 32);
        const int c = small ? (int)((unsigned)i % (unsigned)C) : (int)(i % C);
        const long long p = small ? (long long)((unsigned)i / (unsigned)C) : i / C;
        float d = dOut[p * ld_dout + c_off + c];
        if (act && __bfloat162float(act_out[p * ld_act + act_off + c]) < 0.f) d *= 0.1f;
        dPre[i] = d;
    }
}

// Column sums in two fixed-order passes, for C <= 256: block b sums the rows
// of its slice with T = floor(256 / C) C threads, each keeping one column
// (t mod C, since the stride T is a multiple of C), then part[b][c];
// k_colsum_final adds the blocks in order.
__global__ void __launch_bounds__(256) k_colsum_part(const float* __restrict__ X, long long P, int C, long long rows,
                                                     float* __restrict__ part) {
    const int T = (256 / C) * C;
    const long long r0 = (long long)blockIdx.x * rows;
    const long long r1 = min(P, r0 + rows);
    const float* x = X + r0 * C;
    const long long n = (r1 > r0 ? r1 - r0 : 0) * C;
    float s = 0.f;
    if ((int)threadIdx.x < T)
        for (long long j = threadIdx.x; j < n; j += T) s += x[j];
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    if ((int)threadIdx.x < C) {
        float t = 0.f;
        for (int k = threadIdx.x; k < T; k += C) t += sh[k];
        part[(long long)blockIdx.x * C + threadIdx.x] = t;
    }
}

// One warp per column: lane l adds the partials l, l + 32, ... in order, then
// a fixed shuffle tree adds the lanes (the same order on every call).
__global__ void k_colsum_final(const float* __restrict__ part, int nb, int C, float* __restrict__ out) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= C) return;
    float t = 0.f;
    for (int b = lane; b < nb; b += 32) t += part[(long long)b * C + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[c] = t;
}

// db[c] = sum_p dPre[p][c]: one block per channel group, fixed order.
__global__ void k_colsum(const float* __restrict__ X, long long P, int C, float* __restrict__ out) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (long long p = threadIdx.x; p < P; p += blockDim.x) s += X[p * C + c];
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = sh[0];
}

__global__ void k_pool_fwd(const bf16* __restrict__ X, int Bn, int H, int W, int C, bf16* __restrict__ Y) {
    const int Ho = H / 2, Wo = W / 2;
    const long long total = (long long)Bn * Ho * Wo * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const int x = (int)(p % Wo), y = (int)((p / Wo) % Ho);
        const long long b = p / ((long long)Wo * Ho);
        const bf16* s = X + ((b * H + 2 * y) * W + 2 * x) * C + c;
        const float v = __bfloat162float(s[0]) + __bfloat162float(s[C]) + __bfloat162float(s[(long long)W * C]) +
                        __bfloat162float(s[(long long)W * C + C]);
        Y[i] = __float2bfloat16(0.25f * v);
    }
}

__global__ void k_pool_bwd(const float* __restrict__ dY, int Bn, int H, int W, int C, float* __restrict__ dX) {
    const long long total = (long long)Bn * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        dX[i] = 0.25f * dY[((b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
    }
}

// Nearest 2x upsampling of X [Bn][H][W][C] into a channel slice of Y
// [Bn][2H][2W][ldy] at c_off.
__global__ void k_up_fwd(const bf16* __restrict__ X, int Bn, int H, int W, int C, bf16* __restrict__ Y, int ldy,
                         int c_off) {
    const long long total = (long long)Bn * 4 * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const int x = (int)(p % (2 * W)), y = (int)((p / (2 * W)) % (2 * H));
        const long long b = p / (4LL * W * H);
        Y[p * ldy + c_off + c] = X[((b * H + y / 2) * W + x / 2) * C + c];
    }
}

__global__ void k_up_bwd(const float* __restrict__ dY, int ldy, int c_off, int Bn, int H, int W, int C,
                         float* __restrict__ dX) {
    const long long total = (long long)Bn * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const int x = (int)(p % W), y = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long po = (b * 2 * H + 2 * y + q / 2) * 2 * W + 2 * x + q % 2;
            s += dY[po * ldy + c_off + c];
        }
        dX[i] = s;
    }
}

// Copy a channel slice: dst[p][d_off + c] (ld_dst) = src[p][s_off + c] (ld_src), c < C.
template <class T, class U>
__global__ void k_slice(const T* __restrict__ src, int ld_src, int s_off, long long P, int C, U* __restrict__ dst,
                        int ld_dst, int d_off, int accumulate) {
    const long long total = P * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long p = i / C;
        const float v = (float)src[p * ld_src + s_off + c];
        U* o = dst + p * ld_dst + d_off + c;
        *o = (U)(accumulate ? (float)*o + v : v);
    }
}

// Masked mean-squared error over C channels: weight[p] in {0, 1}.
// dPred = 2 w (pred - target) / (sum w * C); partial sums of w (pred - target)^2.
__global__ void k_mse(const float* __restrict__ pred, const float* __restrict__ target, const float* __restrict__ wgt,
                      long long P, int C, float inv_count, float* __restrict__ dpred, float* __restrict__ part) {
    float s = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P * C;
         i += (long long)gridDim.x * blockDim.x) {
        const float w = wgt[i / C];
        const float d = pred[i] - target[i];
        s += w * d * d;
        dpred[i] = 2.f * w * d * inv_count;
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam (decoupled from the BF16 copies, which mph_nn_cast refreshes) on FP32
// master weights, with L2 weight decay wd.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, float wd, float gscale) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = gscale * grad[i] + wd * w[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

template <class T, class U>
__global__ void k_cast(const T* __restrict__ x, long long n, U* __restrict__ y) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = (U)(float)x[i];
}

// Y[c][r] = X[r][c] for a rows x cols BF16 matrix, through 32 x 32 tiles in
// shared memory (coalesced reads along c and writes along r).  Puts the
// pixel-major operands of a weight gradient (dY [P][Cout], Xcol [P][9 Cin])
// into the K-contiguous layout of the tensor-core GEMM's asynchronous copies.
__global__ void __launch_bounds__(256) k_transpose_bf16(const unsigned short* __restrict__ X, long long rows, int cols,
                                                        unsigned short* __restrict__ Y) {
    __shared__ unsigned short t[32][33];
    const long long r0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        const long long r = r0 + ty + i;
        const int c = c0 + tx;
        if (r < rows && c < cols) t[ty + i][tx] = X[r * cols + c];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 32; i += 8) {
        const int c = c0 + ty + i;
        const long long r = r0 + tx;
        if (r < rows && c < cols) Y[(long long)c * rows + r] = t[tx][ty + i];
    }
}

// The same for even rows and cols through 64 x 64 tiles moved as 32-bit words
// (two BF16 values): a warp reads 128 B of an input row and writes 128 B of an
// output row.  The tile is kept as 16-bit values with rows padded to an odd
// number of words.
__global__ void __launch_bounds__(256) k_transpose_bf16_w(const unsigned* __restrict__ X, long long rows, int cols,
                                                          unsigned* __restrict__ Y) {
    __shared__ unsigned short t[64][66];
    const long long r0 = (long long)blockIdx.x * 64;
    const int c0 = blockIdx.y * 64;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // 8 warps
    const int hc = cols >> 1;                                     // words per input row
    const long long hr = rows >> 1;                               // words per output row
#pragma unroll
    for (int i = 0; i < 64; i += 8) {
        const long long r = r0 + warp + i;
        const int wc = (c0 >> 1) + lane;
        unsigned v = 0u;
        if (r < rows && wc < hc) v = X[r * hc + wc];
        t[warp + i][2 * lane] = (unsigned short)(v & 0xFFFFu);
        t[warp + i][2 * lane + 1] = (unsigned short)(v >> 16);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 64; i += 8) {
        const int c = c0 + warp + i;
        const long long wr = (r0 >> 1) + lane;
        if (c < cols && wr < hr)
            Y[(long long)c * hr + wr] = (unsigned)t[2 * lane][warp + i] | ((unsigned)t[2 * lane + 1][warp + i] << 16);
    }
}

// W2[ci][t Cout + co] = Wt[co][(8 - t) Cin + ci]: the weights of the data
// gradient of a 3 x 3 convolution written as a convolution of dY with the
// taps mirrored (t' = 8 - t) and the channel roles exchanged.
__global__ void k_wflip(const unsigned short* __restrict__ Wt, int cout, int cin, unsigned short* __restrict__ W2) {
    const long long n = 9LL * cout * cin;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int co = (int)(i % cout);
        const long long r = i / cout;
        const int t = (int)(r % 9);
        const int ci = (int)(r / 9);
        W2[i] = Wt[(long long)co * 9 * cin + (long long)(8 - t) * cin + ci];
    }
}

// Block sums of x^2 into part[blockIdx.x].
__global__ void k_sumsq(const float* __restrict__ x, long long n, float* __restrict__ part) {
    float s = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += x[i] * x[i];
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_fill(float* __restrict__ x, long long n, float v) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = v;
}

int grid_for(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    if (b < 1) b = 1;
    return (int)b;
}

int ck(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("nn ") + what + ": " + cudaGetErrorString(e));
    return MPH_OK;
}

}  // namespace

// cuTensorMapEncodeTiled from the driver (through the runtime's entry-point
// query, so the library does not link libcuda); null when unavailable.
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static bool g_encode_tried = false;

static bool tma_available() {
    if (!g_encode_tried) {
        g_encode_tried = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess && fn)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    }
    return g_encode != nullptr;
}

// Map of a row-major BF16 matrix [rows][cols] (row stride ld elements) read
// in boxes of 64 columns (128 B, the swizzle span) x box_rows rows.
static bool tma_map(CUtensorMap* m, const void* ptr, long long rows, long long cols, long long ld, int box_rows,
                    int box_cols = 64) {
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1u, 1u};
    return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, box_cols == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Map of an NHWC BF16 activation [B][H][W][C] as the 4-D tensor (C, W, H, B),
// read in boxes of bkc channels x a 128-pixel piece (bw pixels of bh rows).
static bool tma_map_act(CUtensorMap* m, const void* ptr, int Bn, int H, int W, int C, int bkc, int bw, int bh) {
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)Bn};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)bkc, (cuuint32_t)bw, (cuuint32_t)bh, 1u};
    const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
    return g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(ptr), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, bkc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Per-device state of the surrogate kernels (the workspaces live on the
// device that was current when they were made).
constexpr int kMaxDevices = 64;

static int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return -1;
    return d;
}

template <int BN, int BKC = 64, bool CONV = false>
static cudaError_t launch_tma(const dim3& g, int M, int N, const CUtensorMap& ta, const CUtensorMap& tb, float* out,
                              long long ldo, int acc, int K, int kchunk, cudaStream_t s, ConvGeom cg = ConvGeom{}) {
    static unsigned long long attr_set = 0;  // bit d: the shared-memory limit is raised on device d
    constexpr size_t smem = tma_smem_bytes<BN, BKC>();
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    if (!(attr_set >> dev & 1ull)) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_gemm_tma<BN, BKC, CONV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set |= 1ull << dev;
    }
    k_gemm_tma<BN, BKC, CONV><<<g, 128, smem, s>>>(M, N, ta, tb, out, ldo, acc, K, kchunk, cg);
    return cudaGetLastError();
}

extern "C" {

int mph_nn_alloc(long long bytes, void** out) {
    if (!out || bytes <= 0) return mph::fail(MPH_ERR_ARG, "mph_nn_alloc: bad argument");
    const cudaError_t e = cudaMalloc(out, (size_t)bytes);
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_alloc: ") + cudaGetErrorString(e));
    return MPH_OK;
}

int mph_nn_free(void* p) {
    cudaFree(p);
    return MPH_OK;
}

// dir: 0 = host -> device, 1 = device -> host, 2 = device -> device.
int mph_nn_copy(void* dst, const void* src, long long bytes, int dir, void* stream) {
    const cudaMemcpyKind k = dir == 0 ? cudaMemcpyHostToDevice : (dir == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
    cudaError_t e = cudaMemcpyAsync(dst, src, (size_t)bytes, k, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess && dir != 2) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_copy: ") + cudaGetErrorString(e));
    return MPH_OK;
}

int mph_nn_sync(void* stream) {
    const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_sync: ") + cudaGetErrorString(e));
    return MPH_OK;
}

// 0 auto, 1 mma.sync, 2 tcgen05 pipelined (cp.async), 3 tcgen05 single-
// buffered, 4 tcgen05 fed by TMA (where both operands are K-contiguous and
// 16-byte aligned; the pipelined kernel otherwise)
static int g_gemm_mode = 0;

int mph_nn_gemm_mode(int mode) {
    if (mode < 0 || mode > 4)
        return mph::fail(MPH_ERR_ARG, "mph_nn_gemm_mode: 0 auto, 1 mma.sync, 2 tcgen05, 3 tcgen05 single-buffered, "
                                      "4 tcgen05 with TMA");
    g_gemm_mode = mode;
    return MPH_OK;
}

int mph_nn_status(int* timeout, int reset) {
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_nn_timeout, sizeof(int));
    if (e == cudaSuccess && reset) {
        const int z = 0;
        e = cudaMemcpyToSymbol(g_nn_timeout, &z, sizeof(int));
    }
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_status: ") + cudaGetErrorString(e));
    if (timeout) *timeout = v;
    return MPH_OK;
}

// Split-K workspace, grown on demand (the weight gradients have a small
// output and K = the pixel count).
// One per device.
static float* g_ws_dev[kMaxDevices] = {};
static size_t g_ws_bytes_dev[kMaxDevices] = {};

// Enough blocks for the 152 SMs: split K (in multiples of 64) when the
// output tiles are few.
static void split_plan(long long blocks, int K, int& S, int& kchunk) {
    S = 1;
    kchunk = K;
    if (blocks < 2 * 152 && K >= 8 * 64) {
        S = (int)std::min<long long>((2 * 152 + blocks - 1) / blocks, K / (4 * 64));
        S = std::max(1, std::min(S, 64));
        kchunk = (K + S - 1) / S;
        kchunk = (kchunk + 63) / 64 * 64;
        S = (K + kchunk - 1) / kchunk;
    }
}

// The split-K workspace of the current device, grown to `need` bytes.
static int split_workspace(size_t need, float** ws, const char* who) {
    const int dev = current_device();
    if (dev < 0) return mph::fail(MPH_ERR_CUDA, std::string(who) + ": no current device");
    if (need > g_ws_bytes_dev[dev]) {
        cudaFree(g_ws_dev[dev]);
        g_ws_dev[dev] = nullptr;
        g_ws_bytes_dev[dev] = 0;
        const cudaError_t e = cudaMalloc(&g_ws_dev[dev], need);
        if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string(who) + " workspace: " + cudaGetErrorString(e));
        g_ws_bytes_dev[dev] = need;
    }
    *ws = g_ws_dev[dev];
    return MPH_OK;
}

static void splitk_reduce(const float* ws, int S, int M, int N, float* C, long long ldc, int accumulate,
                          cudaStream_t s) {
    const long long total = (long long)M * N;
    if (S > 4) k_splitk_reduce4<<<(unsigned)((total + 63) / 64), 256, 0, s>>>(ws, S, M, N, C, ldc, accumulate);
    else k_splitk_reduce<<<grid_for(total), 256, 0, s>>>(ws, S, M, N, C, ldc, accumulate);
}

int mph_nn_gemm(int M, int N, int K, const void* A, long long lda, int ta, const void* B, long long ldb, int tb,
                float* C, long long ldc, int accumulate, void* stream) {
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C) return mph::fail(MPH_ERR_ARG, "mph_nn_gemm: bad argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto a = static_cast<const bf16*>(A);
    auto b = static_cast<const bf16*>(B);
    // tcgen05 tiles are 128 rows: below that the mma.sync kernel, unless K
    // is long (a weight gradient, K = pixels), where the idle rows cost less
    // than the slower kernel.
    const bool tc = g_gemm_mode >= 2 || (g_gemm_mode == 0 && (M >= TC_BM || K >= 16 * TC_BK) && N >= 16);
    // TMA operands: K-contiguous, 16-byte aligned bases and row strides
    const bool tma = tc && (g_gemm_mode == 0 || g_gemm_mode == 4) && !ta && !tb &&
                     ((reinterpret_cast<unsigned long long>(A) | reinterpret_cast<unsigned long long>(B)) & 15) == 0 &&
                     lda % 8 == 0 && ldb % 8 == 0 && tma_available();
    const int tma_bn = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
    const int tm = tc ? TC_BM : BM, tn = tma ? tma_bn : (tc ? TC_BN : BN);
    const long long gx = (N + tn - 1) / tn, gy = (M + tm - 1) / tm;
    if (gy > 65535) return mph::fail(MPH_ERR_ARG, "mph_nn_gemm: M too large for one launch");
    int S = 1, kchunk = K;
    split_plan(gx * gy, K, S, kchunk);
    float* out = C;
    long long ldo = ldc;
    int acc = accumulate;
    float* ws = nullptr;
    if (S > 1) {
        const int rc = split_workspace((size_t)S * M * N * sizeof(float), &ws, "mph_nn_gemm");
        if (rc) return rc;
        out = ws;
        ldo = N;
        acc = 0;
    }
    const dim3 g((unsigned)gx, (unsigned)gy, (unsigned)S);
    if (tma) {
        CUtensorMap tA, tB;
        if (!tma_map(&tA, A, M, K, lda, 128) || !tma_map(&tB, B, N, K, ldb, tma_bn))
            return mph::fail(MPH_ERR_CUDA, "mph_nn_gemm: cuTensorMapEncodeTiled failed");
        cudaError_t e = tma_bn == 32 ? launch_tma<32>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s)
                      : tma_bn == 64 ? launch_tma<64>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s)
                                     : launch_tma<128>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s);
        if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_gemm (TMA): ") + cudaGetErrorString(e));
        if (S > 1) splitk_reduce(ws, S, M, N, C, ldc, accumulate, s);
        return ck("gemm (tcgen05, TMA)");
    }
#define MPH_GEMM_LAUNCH(KERN)                                                                                  \
    if (!ta && !tb) KERN<false, false><<<g, 128, 0, s>>>(M, N, K, a, lda, b, ldb, out, ldo, acc, kchunk);      \
    else if (!ta && tb) KERN<false, true><<<g, 128, 0, s>>>(M, N, K, a, lda, b, ldb, out, ldo, acc, kchunk);   \
    else if (ta && !tb) KERN<true, false><<<g, 128, 0, s>>>(M, N, K, a, lda, b, ldb, out, ldo, acc, kchunk);   \
    else KERN<true, true><<<g, 128, 0, s>>>(M, N, K, a, lda, b, ldb, out, ldo, acc, kchunk);
    if (tc && g_gemm_mode == 3) {
        MPH_GEMM_LAUNCH(k_gemm_tc05)
    } else if (tc) {
        MPH_GEMM_LAUNCH(k_gemm_tc05p)
    } else {
        MPH_GEMM_LAUNCH(k_gemm_bf16)
    }
#undef MPH_GEMM_LAUNCH
    if (S > 1) splitk_reduce(ws, S, M, N, C, ldc, accumulate, s);
    return ck(tc ? "gemm (tcgen05)" : "gemm (mma.sync)");
}

// Y[p][co] (+)= sum over taps t and channels c of X[pixel p shifted by t][c]
// Wt[co][t C + c]: the forward GEMM of a 3 x 3, pad 1 convolution without the
// im2col matrix (k_gemm_tma<BN, BKC, true>).  MPH_ERR_UNSUPPORTED when the
// shapes do not fit the implicit kernel (C not a multiple of 32, image rows
// that do not tile 128-pixel blocks, unaligned buffers, no TMA); the caller
// then uses im2col + mph_nn_gemm.
int mph_nn_conv3(const void* X, int Bn, int H, int W, int C, const void* Wt, int Cout, float* Y, int accumulate,
                 void* stream) {
    if (!X || !Wt || !Y || Bn <= 0 || H <= 0 || W <= 0 || C <= 0 || Cout <= 0)
        return mph::fail(MPH_ERR_ARG, "mph_nn_conv3: bad argument");
    const long long P = (long long)Bn * H * W;
    const int bw = W < 128 ? W : 128, bh = 128 / bw;
    const bool tiles = W >= 128 ? W % 128 == 0 : (128 % W == 0 && H % bh == 0);
    const bool aligned = ((reinterpret_cast<unsigned long long>(X) | reinterpret_cast<unsigned long long>(Wt)) & 15) == 0;
    if (C % 32 != 0 || !tiles || P % 128 != 0 || P / 128 > 65535 || !aligned || (long long)9 * C > 0x7fffffffLL ||
        !tma_available())
        return mph::fail(MPH_ERR_UNSUPPORTED, "mph_nn_conv3: shapes outside the implicit-GEMM kernel");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int bkc = C % 64 == 0 ? 64 : 32;
    const int M = (int)P, N = Cout, K = 9 * C;
    const int bn = N <= 32 ? 32 : (N <= 64 ? 64 : 128);
    const long long gx = (N + bn - 1) / bn, gy = P / 128;
    int S = 1, kchunk = K;
    split_plan(gx * gy, K, S, kchunk);
    float* out = Y;
    long long ldo = N;
    int acc = accumulate;
    float* ws = nullptr;
    if (S > 1) {
        const int rc = split_workspace((size_t)S * M * N * sizeof(float), &ws, "mph_nn_conv3");
        if (rc) return rc;
        out = ws;
        acc = 0;
    }
    CUtensorMap tA, tB;
    if (!tma_map_act(&tA, X, Bn, H, W, C, bkc, bw, bh) || !tma_map(&tB, Wt, N, K, K, bn, bkc))
        return mph::fail(MPH_ERR_CUDA, "mph_nn_conv3: cuTensorMapEncodeTiled failed");
    const dim3 g((unsigned)gx, (unsigned)gy, (unsigned)S);
    const ConvGeom cg{C, H, W};
    cudaError_t e;
    if (bkc == 64)
        e = bn == 32 ? launch_tma<32, 64, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg)
          : bn == 64 ? launch_tma<64, 64, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg)
                     : launch_tma<128, 64, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg);
    else
        e = bn == 32 ? launch_tma<32, 32, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg)
          : bn == 64 ? launch_tma<64, 32, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg)
                     : launch_tma<128, 32, true>(g, M, N, tA, tB, out, ldo, acc, K, kchunk, s, cg);
    if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_conv3: ") + cudaGetErrorString(e));
    if (S > 1) splitk_reduce(ws, S, M, N, Y, N, accumulate, s);
    return ck("conv3 (tcgen05, TMA, implicit GEMM)");
}

int mph_nn_im2col3(const void* X, int Bn, int H, int W, int C, void* Xcol, void* stream) {
    const long long n = (long long)Bn * H * W * 9 * C;
    const bool aligned = ((reinterpret_cast<unsigned long long>(X) | reinterpret_cast<unsigned long long>(Xcol)) & 15) == 0;
    if (C % 8 == 0 && aligned && n / 8 < 0xffffffffLL) {
        const long long nv = n / 8;
        k_im2col3_v8<<<(unsigned)((nv + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const uint4*>(X), Bn, H, W, C / 8, static_cast<uint4*>(Xcol));
        return ck("im2col");
    }
    k_im2col3<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(X), Bn, H, W, C,
                                                                           static_cast<bf16*>(Xcol));
    return ck("im2col");
}

int mph_nn_col2im3(const float* dXcol, int Bn, int H, int W, int C, float* dX, void* stream) {
    const long long n = (long long)Bn * H * W * C;
    k_col2im3<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(dXcol, Bn, H, W, C, dX);
    return ck("col2im");
}

int mph_nn_bias_act(const float* Y, const float* bias, long long P, int C, int act, void* out_bf16, float* out_f32,
                    int ld_out, int c_off, void* stream) {
    k_bias_act<<<grid_for(P * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(Y, bias, P, C, act,
                                                                               static_cast<bf16*>(out_bf16), out_f32,
                                                                               ld_out, c_off);
    return ck("bias_act");
}

int mph_nn_act_bwd(const float* dOut, int ld_dout, int c_off, const void* act_out, int ld_act, int act_off,
                   long long P, int C, int act, float* dPre, void* stream) {
    k_act_bwd<<<grid_for(P * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        dOut, ld_dout, c_off, static_cast<const bf16*>(act_out), ld_act, act_off, P, C, act, dPre);
    return ck("act_bwd");
}

// [blocks][C] partial column sums, shared by every call: calls on different
// streams must not overlap (the surrogate issues all its kernels on one stream).
static float* g_colsum_ws[kMaxDevices] = {};
static constexpr int kColsumBlocks = 608;

int mph_nn_colsum(const float* X, long long P, int C, float* out, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (C > 0 && C <= 256 && P >= 256) {
        const int dev = current_device();
        if (dev < 0) return mph::fail(MPH_ERR_CUDA, "mph_nn_colsum: no current device");
        if (!g_colsum_ws[dev]) {
            const cudaError_t e = cudaMalloc(&g_colsum_ws[dev], sizeof(float) * kColsumBlocks * 256);
            if (e != cudaSuccess) return mph::fail(MPH_ERR_CUDA, std::string("mph_nn_colsum: ") + cudaGetErrorString(e));
        }
        float* ws = g_colsum_ws[dev];
        const long long rows = (P + kColsumBlocks - 1) / kColsumBlocks;
        const int nb = (int)((P + rows - 1) / rows);
        k_colsum_part<<<nb, 256, 0, s>>>(X, P, C, rows, ws);
        k_colsum_final<<<(C + 7) / 8, 256, 0, s>>>(ws, nb, C, out);
        return ck("colsum");
    }
    k_colsum<<<C, 256, 0, s>>>(X, P, C, out);
    return ck("colsum");
}

int mph_nn_pool(const void* X, int Bn, int H, int W, int C, void* Y, void* stream) {
    const long long n = (long long)Bn * (H / 2) * (W / 2) * C;
    k_pool_fwd<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(X), Bn, H, W, C,
                                                                            static_cast<bf16*>(Y));
    return ck("pool");
}

int mph_nn_pool_bwd(const float* dY, int Bn, int H, int W, int C, float* dX, void* stream) {
    k_pool_bwd<<<grid_for((long long)Bn * H * W * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(dY, Bn, H, W, C, dX);
    return ck("pool_bwd");
}

int mph_nn_up(const void* X, int Bn, int H, int W, int C, void* Y, int ldy, int c_off, void* stream) {
    k_up_fwd<<<grid_for(4LL * Bn * H * W * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(X), Bn, H, W, C, static_cast<bf16*>(Y), ldy, c_off);
    return ck("up");
}

int mph_nn_up_bwd(const float* dY, int ldy, int c_off, int Bn, int H, int W, int C, float* dX, void* stream) {
    k_up_bwd<<<grid_for((long long)Bn * H * W * C), 256, 0, static_cast<cudaStream_t>(stream)>>>(dY, ldy, c_off, Bn, H,
                                                                                                  W, C, dX);
    return ck("up_bwd");
}

// kind: 0 = bf16 -> bf16, 1 = f32 -> f32 (accumulate allowed), 2 = f32 -> bf16.
int mph_nn_slice(int kind, const void* src, int ld_src, int s_off, long long P, int C, void* dst, int ld_dst,
                 int d_off, int accumulate, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int g = grid_for(P * C);
    if (kind == 0)
        k_slice<bf16, bf16><<<g, 256, 0, s>>>(static_cast<const bf16*>(src), ld_src, s_off, P, C,
                                              static_cast<bf16*>(dst), ld_dst, d_off, 0);
    else if (kind == 1)
        k_slice<float, float><<<g, 256, 0, s>>>(static_cast<const float*>(src), ld_src, s_off, P, C,
                                                static_cast<float*>(dst), ld_dst, d_off, accumulate);
    else
        k_slice<float, bf16><<<g, 256, 0, s>>>(static_cast<const float*>(src), ld_src, s_off, P, C,
                                               static_cast<bf16*>(dst), ld_dst, d_off, 0);
    return ck("slice");
}

int mph_nn_mse(const float* pred, const float* target, const float* wgt, long long P, int C, float inv_count,
               float* dpred, float* part, int nblocks, void* stream) {
    k_mse<<<nblocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(pred, target, wgt, P, C, inv_count, dpred, part);
    return ck("mse");
}

int mph_nn_adam(float* w, float* m, float* v, const float* grad, long long n, float lr, float b1, float b2, float eps,
                int t, float wd, float gscale, void* stream) {
    const float c1 = 1.f / (1.f - powf(b1, (float)t)), c2 = 1.f / (1.f - powf(b2, (float)t));
    k_adam<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, m, v, grad, n, lr, b1, b2, eps, c1, c2, wd,
                                                                         gscale);
    return ck("adam");
}

int mph_nn_sumsq(const float* x, long long n, float* part, int nblocks, void* stream) {
    k_sumsq<<<nblocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, part);
    return ck("sumsq");
}

// kind: 0 = f32 -> bf16, 1 = bf16 -> f32.
int mph_nn_cast(int kind, const void* x, long long n, void* y, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (kind == 0) k_cast<float, bf16><<<grid_for(n), 256, 0, s>>>(static_cast<const float*>(x), n, static_cast<bf16*>(y));
    else k_cast<bf16, float><<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(x), n, static_cast<float*>(y));
    return ck("cast");
}

int mph_nn_transpose(const void* x, long long rows, int cols, void* y, void* stream) {
    if (!x || !y || rows <= 0 || cols <= 0 || (rows + 31) / 32 > 0x7fffffffLL || (cols + 31) / 32 > 65535)
        return mph::fail(MPH_ERR_ARG, "mph_nn_transpose: bad argument");
    const bool words = rows % 2 == 0 && cols % 2 == 0 &&
                       ((reinterpret_cast<unsigned long long>(x) | reinterpret_cast<unsigned long long>(y)) & 3) == 0;
    if (words && (rows + 63) / 64 <= 0x7fffffffLL && (cols + 63) / 64 <= 65535) {
        const dim3 grid((unsigned)((rows + 63) / 64), (unsigned)((cols + 63) / 64));
        k_transpose_bf16_w<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const unsigned*>(x), rows,
                                                                                cols, static_cast<unsigned*>(y));
        return ck("transpose");
    }
    const dim3 grid((unsigned)((rows + 31) / 32), (unsigned)((cols + 31) / 32));
    k_transpose_bf16<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const unsigned short*>(x), rows,
                                                                          cols, static_cast<unsigned short*>(y));
    return ck("transpose");
}

int mph_nn_wflip(const void* wt, int cout, int cin, void* w2, void* stream) {
    if (!wt || !w2 || cout <= 0 || cin <= 0) return mph::fail(MPH_ERR_ARG, "mph_nn_wflip: bad argument");
    const long long n = 9LL * cout * cin;
    k_wflip<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const unsigned short*>(wt), cout, cin,
                                                                        static_cast<unsigned short*>(w2));
    return ck("wflip");
}

int mph_nn_fill(float* x, long long n, float v, void* stream) {
    k_fill<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, v);
    return ck("fill");
}

}  // extern "C"
