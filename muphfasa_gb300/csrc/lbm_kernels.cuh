// lbm_kernels.cuh -- device code of the fused lattice-Boltzmann step.
//
// One thread owns one cell.  A step pulls the Q populations that stream into
// the cell (f_in(x - c_n, n), Streaming.H:20-35), takes the moments, relaxes
// towards equilibrium (BGK, with the Guo force term when forced) and writes Q
// populations: 2*Q*sizeof(T) bytes of HBM traffic per cell update, no ghost
// layer.  Boundaries are applied link-wise inside the pull: a population
// whose upstream cell g = x - c_n lies outside the domain in a non-periodic
// direction takes the value that the reference's ghost fill would have
// written at g (BCManager<L>::operator(), BoundaryConditions.H:124-189), and
// that value depends only on the post-collision populations of x itself
// because the ghost-fill source cell is g + c_n = x.  Periodic directions
// wrap the index, which equals the reference's FillBoundary copy.
//
// Two arithmetic modes share the pull:
//   kExact -- the reference's floating-point operation order (Collision.cpp
//             :18-92, Macroscopic.H, Equilibrium.H:28-57, Collision.H:21-76);
//             compiled in a translation unit with --fmad=false it reproduces
//             the reference's FP64 results bit for bit.
//   kFast  -- algebraically refactored, FMA-contracted arithmetic (pair
//             sums for the moments, one reciprocal, shared quadratic terms)
//             in the compute type R of the storage policy.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lattice.cuh"

namespace mph {

enum { kBcMoving = 0, kBcNoSlip = 1, kBcInflow = 2, kBcOutflow = 3, kBcPressure = 4, kBcPeriodic = 5 };
enum { kExact = 0, kFast = 1 };
enum { kFluid = 0, kNearSolid = 1, kSolid = 2 };

// Per-domain constants passed by value to every kernel.
struct KParams {
    int nx, ny, nz;
    int periodic[3];
    long long ncell;      // nx*ny*nz: stride between populations
    double omega, omc;    // omega and 1 - omega (BGK::collide, Collision.H:68-76)
    double F[3], hF[3];   // body force and 0.5*F (Macroscopic.H:241-278)
    double gpref[27];     // ((1 - 0.5 omega) w_n) cs2inv  (guoForceTerm prefactor)
    double gcF[27];       // c_n . F                         (guoForceTerm)
    int bc_type[27];      // resolved ghost-class table (BCManager::finalize)
    double bc_rho[27];
    double bc_U[27][3];
    // FP32 copies for the single-precision collide: a double->float
    // conversion runs on the FP64 pipe (2 per SM per clock on GB300).
    float omega_f, hF_f[3], F_f[3], gpref_f[27], gcF_f[27];
    float inv_nx_f, inv_ny_f;  // 1/nx, 1/ny (cell coordinates in the batch kernel)
    // Interior obstacles (no counterpart in the reference): one class byte per
    // cell, kFluid / kNearSolid (a fluid cell with a solid upstream cell) /
    // kSolid; nullptr when the domain has none (no extra traffic then).
    const unsigned char* cls;
    // Window of one step launch: rows [y0, y1) of planes [z0, z1).  The full
    // domain is (0, ny, 0, nz); a host-copy pipeline steps slabs of planes.
    int y0, y1, z0, z1;
    // Status flag of the handle for storages whose stores can saturate
    // (StF16W sets bit 4); nullptr otherwise.
    int* flag;
};

// Parameters in the compute type R of a collide.
template <class R> struct Prm;
template <> struct Prm<double> {
    static __device__ __forceinline__ double omega(const KParams& p) { return p.omega; }
    static __device__ __forceinline__ double hF(const KParams& p, int a) { return p.hF[a]; }
    static __device__ __forceinline__ double F(const KParams& p, int a) { return p.F[a]; }
    static __device__ __forceinline__ double gpref(const KParams& p, int n) { return p.gpref[n]; }
    static __device__ __forceinline__ double gcF(const KParams& p, int n) { return p.gcF[n]; }
};
template <> struct Prm<float> {
    static __device__ __forceinline__ float omega(const KParams& p) { return p.omega_f; }
    static __device__ __forceinline__ float hF(const KParams& p, int a) { return p.hF_f[a]; }
    static __device__ __forceinline__ float F(const KParams& p, int a) { return p.F_f[a]; }
    static __device__ __forceinline__ float gpref(const KParams& p, int n) { return p.gpref_f[n]; }
    static __device__ __forceinline__ float gcF(const KParams& p, int n) { return p.gcF_f[n]; }
};

// Extra constants of the fixed-point step (k_f64x.cu).
struct KParamsX {
    unsigned long long W;      // omega / 2 in Q0.64, low bit clear
    unsigned long long wh1;    // W / 2 - 1 (rounding constant of the omega multiply)
    unsigned long long Wm;     // 32 x the smallest lattice weight in Q0.64
    long long hF[3];           // F / 2 in Q.56
    long long Fw[3];           // 3 (1 - omega/2) F / omega in Q.56 (Guo term over omega)
    int fmask;                 // bit b set when Fw[b] != 0
};

// ---------------------------------------------------------------------------
// Storage policies: how a population is kept in HBM and the compute type R.
// ---------------------------------------------------------------------------
struct StF64 {
    using T = double;
    static constexpr bool kShift = false;
    static constexpr bool kPerPop = false, kRange = false;
    using R = double;
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int, unsigned e) { return __ldg(f + e); }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int, unsigned e, R v) { f[e] = v; }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return __ldg(f + n * N + i);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = v;
    }
    // Value that a store followed by a load returns.
    template <int Q> static __device__ __forceinline__ R rt(int, R v) { return v; }
};
struct StF32 {
    using T = float;
    static constexpr bool kShift = false;
    static constexpr bool kPerPop = false, kRange = false;
    using R = float;
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int, unsigned e) { return __ldg(f + e); }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int, unsigned e, R v) { f[e] = v; }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return __ldg(f + n * N + i);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = v;
    }
    template <int Q> static __device__ __forceinline__ R rt(int, R v) { return v; }
};
// Shifted 16-bit storage: the deviation f_n - w_n is stored, so that the
// 11 (FP16) or 8 (BF16) significant bits resolve the small departure from the
// rest state instead of the O(w) value itself.
struct StF16S {
    using T = __half;
    using R = float;
    // Shifted kernels work on g = f - w directly: one value (ldr1/str1) or an
    // aligned pair of neighbouring cells (ldr2/str2, e even).
    static constexpr bool kShift = true;
    static constexpr bool kPerPop = false, kRange = false;
    static __device__ __forceinline__ float ldr1(const T* __restrict__ f, unsigned e) { return __half2float(f[e]); }
    static __device__ __forceinline__ float2 ldr2(const T* __restrict__ f, unsigned e) {
        return __half22float2(*reinterpret_cast<const __half2*>(f + e));
    }
    // the same conversions from raw bits (values staged in shared memory)
    static __device__ __forceinline__ float dec1(unsigned h) { return __half2float(__ushort_as_half((unsigned short)h)); }
    static __device__ __forceinline__ float2 dec2(unsigned w) {
        return __half22float2(__halves2half2(__ushort_as_half((unsigned short)(w & 0xFFFFu)),
                                             __ushort_as_half((unsigned short)(w >> 16))));
    }
    static __device__ __forceinline__ void str1(T* __restrict__ f, unsigned e, float v) { f[e] = __float2half_rn(v); }
    static __device__ __forceinline__ void str2(T* __restrict__ f, unsigned e, float2 v) {
        *reinterpret_cast<__half2*>(f + e) = __floats2half2_rn(v.x, v.y);
    }
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int n, unsigned e) {
        return __half2float(f[e]) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int n, unsigned e, R v) {
        f[e] = __float2half_rn(v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return __half2float(f[n * N + i]) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = __float2half_rn(v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R rt(int n, R v) {
        return __half2float(__float2half_rn(v - (float)Lat<Q>::w(n))) + (float)Lat<Q>::w(n);
    }
};
struct StBF16S {
    using T = __nv_bfloat16;
    using R = float;
    static constexpr bool kShift = true;
    static constexpr bool kPerPop = false, kRange = false;
    // bf16 is the high half of an FP32 word: widening is a shift / mask.
    static __device__ __forceinline__ float ldr1(const T* __restrict__ f, unsigned e) {
        return __uint_as_float((unsigned)__ldg(reinterpret_cast<const unsigned short*>(f) + e) << 16);
    }
    static __device__ __forceinline__ float dec1(unsigned h) { return __uint_as_float(h << 16); }
    static __device__ __forceinline__ float2 dec2(unsigned w) {
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
    }
    static __device__ __forceinline__ float2 ldr2(const T* __restrict__ f, unsigned e) {
        return dec2(__ldg(reinterpret_cast<const unsigned*>(f + e)));
    }
    static __device__ __forceinline__ void str1(T* __restrict__ f, unsigned e, float v) { f[e] = __float2bfloat16_rn(v); }
    static __device__ __forceinline__ void str2(T* __restrict__ f, unsigned e, float2 v) {
        *reinterpret_cast<__nv_bfloat162*>(f + e) = __floats2bfloat162_rn(v.x, v.y);
    }
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int n, unsigned e) {
        return __bfloat162float(f[e]) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int n, unsigned e, R v) {
        f[e] = __float2bfloat16_rn(v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return __bfloat162float(f[n * N + i]) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = __float2bfloat16_rn(v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R rt(int n, R v) {
        return __bfloat162float(__float2bfloat16_rn(v - (float)Lat<Q>::w(n))) + (float)Lat<Q>::w(n);
    }
};

// Shifted custom 16-bit float (MPH_PREC_F16C): the deviation f_n - w_n in a
// 1-4-11 format (sign, 4 exponent bits with bias 16, 11 stored mantissa
// bits), after the custom FP16 formats for lattice-Boltzmann populations of
// Lehmann et al., Phys. Rev. E 106, 015308 (2022): the deviations stay far
// below 1, so IEEE FP16's upper exponent range is traded for a 12-bit
// significand (half the rounding error of FP16).  Normals span 2^-15 up to
// 1 - 2^-12, subnormals reach down in steps of 2^-26; magnitudes from
// 1 - 2^-13 up saturate at the largest value.  Conversions are bit
// arithmetic around one power-of-two FP32
// multiply (no denormal flushing in these translation units):
//   decode: the 15 magnitude bits placed at FP32 bit 12 read as an FP32
//           number 2^(e-127)(1 + m/2^11) (or an FP32 subnormal for e = 0);
//           times 2^(127-16) rebias it, subnormals included;
//   encode: times 2^(16-127), then round the FP32 bits to nearest even at
//           bit 12 (carries run into the exponent as they should).
namespace f16c {
__device__ __forceinline__ float decode(unsigned h) {
    const unsigned u = ((h & 0x8000u) << 16) | ((h & 0x7FFFu) << 12);
    return __fmul_rn(__uint_as_float(u), 0x1p111f);
}
__device__ __forceinline__ unsigned encode(float x) {
    const unsigned u = __float_as_uint(__fmul_rn(x, 0x1p-111f));
    const unsigned a = u & 0x7FFFFFFFu;
    unsigned r = (a + 0x7FFu + ((a >> 12) & 1u)) >> 12;
    r = r > 0x7FFFu ? 0x7FFFu : r;
    return ((u >> 16) & 0x8000u) | r;
}
}  // namespace f16c

struct StF16C {
    using T = unsigned short;
    using R = float;
    static constexpr bool kShift = true;
    static constexpr bool kPerPop = false, kRange = false;
    static __device__ __forceinline__ float ldr1(const T* __restrict__ f, unsigned e) { return f16c::decode(__ldg(f + e)); }
    static __device__ __forceinline__ float dec1(unsigned h) { return f16c::decode(h); }
    static __device__ __forceinline__ float2 dec2(unsigned w) {
        return make_float2(f16c::decode(w & 0xFFFFu), f16c::decode(w >> 16));
    }
    static __device__ __forceinline__ float2 ldr2(const T* __restrict__ f, unsigned e) {
        return dec2(__ldg(reinterpret_cast<const unsigned*>(f + e)));
    }
    static __device__ __forceinline__ void str1(T* __restrict__ f, unsigned e, float v) {
        f[e] = (unsigned short)f16c::encode(v);
    }
    static __device__ __forceinline__ void str2(T* __restrict__ f, unsigned e, float2 v) {
        *reinterpret_cast<unsigned*>(f + e) = f16c::encode(v.x) | (f16c::encode(v.y) << 16);
    }
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int n, unsigned e) {
        return ldr1(f, e) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int n, unsigned e, R v) {
        str1(f, e, v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return ldr1(f, (unsigned)(n * N + i)) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = (unsigned short)f16c::encode(v - (float)Lat<Q>::w(n));
    }
    template <int Q> static __device__ __forceinline__ R rt(int n, R v) {
        return f16c::decode(f16c::encode(v - (float)Lat<Q>::w(n))) + (float)Lat<Q>::w(n);
    }
};

// Shifted, weight-scaled custom 16-bit float (MPH_PREC_F16W): the deviation
// x_n = (f_n - w_n) / p_n, p_n the power of two nearest to w_n (0.75 w_n <=
// p_n <= 1.125 w_n on every lattice), as sign, 3 exponent bits with bias 8
// and 12 stored mantissa bits.  Divided by
// (about) its weight, every population's deviation is of the same size
// (about 3 |c.u| + |rho - 1|), so eight binades of exponent cover the range
// and the bit saved on the exponent goes to the significand: 13 significant
// bits against the 12 of StF16C.  Normals span 2^-7 up to 1 - 2^-13,
// subnormals are multiples of 2^-19 (the resolution of the small deviations
// of the rest and cross-flow populations, which carry the pressure); from
// 1 - 2^-14 up a magnitude saturates at the largest value and the step sets
// bit 2 (value 4) of the handle's flag: every population must stay inside
// (w_n - p_n, w_n + p_n), which holds for |u| up to about 0.1 in any
// direction (a lid at 0.1 included) and fails in an unstable run.
// The scale is a power of two so that decoding inverts encoding exactly: with
// w_n itself, the FP32-rounded w_n times its exact inverse differs from 1 by
// up to 2^-24, and that factor on every deviation compounds step after step
// (measured: a steady kinetic-energy drift of 3e-5 per 1000 steps of a 3-D
// Taylor-Green vortex).  Conversions are bit arithmetic around one FP32
// multiply by a power of two (no denormal flushing in these units):
//   decode: the 15 magnitude bits placed at FP32 bit 11 read as the FP32
//           number 2^(e-127)(1 + m/2^12) (a subnormal for e = 0); times
//           p_n 2^(127-8) it is g_n = f_n - w_n;
//   encode: g_n times 2^(8-127) / p_n, then the FP32 bits rounded to nearest
//           even at bit 11.
namespace f16w {
// log2 p_n by weight class |c_n|^2 (D2Q9 4/9, 1/9, 1/36 -> 1/2, 1/8, 1/32;
// D3Q15 2/9, 1/9, 1/72 -> 1/4, 1/8, 1/64; D3Q19 1/3, 1/18, 1/36 -> 1/4,
// 1/16, 1/32; D3Q27 8/27, 2/27, 1/54, 1/216 -> 1/4, 1/16, 1/64, 1/256).  The
// scales are built from exponent bits, so an unrolled loop over n sees
// immediate constants.
template <int Q> __device__ __forceinline__ constexpr int lp(int n) {
    using L = Lat<Q>;
    const int k = L::cx(n) * L::cx(n) + L::cy(n) * L::cy(n) + L::cz(n) * L::cz(n);
    return Q == 9 ? (k == 0 ? -1 : k == 1 ? -3 : -5)
         : Q == 15 ? (k == 0 ? -2 : k == 1 ? -3 : -6)
         : Q == 19 ? (k == 0 ? -2 : k == 1 ? -4 : -5)
                   : (k == 0 ? -2 : k == 1 ? -4 : k == 2 ? -6 : -8);
}
// p_n 2^119 and 2^-119 / p_n
template <int Q> __device__ __forceinline__ float dscale(int n) { return __int_as_float((lp<Q>(n) + 246) << 23); }
template <int Q> __device__ __forceinline__ float escale(int n) { return __int_as_float((8 - lp<Q>(n)) << 23); }
template <int Q> __device__ __forceinline__ float decode(int n, unsigned h) {
    return __fmul_rn(__uint_as_float(((h & 0x8000u) << 16) | ((h & 0x7FFFu) << 11)), dscale<Q>(n));
}
// sat collects the unclamped magnitude codes: above 0x7FFF a value saturated.
template <int Q> __device__ __forceinline__ unsigned encode(int n, float g, unsigned& sat) {
    const unsigned u = __float_as_uint(__fmul_rn(g, escale<Q>(n)));
    const unsigned a = u & 0x7FFFFFFFu;
    const unsigned r = (a + 0x3FFu + ((a >> 11) & 1u)) >> 11;
    sat |= r;
    return ((u >> 16) & 0x8000u) | (r > 0x7FFFu ? 0x7FFFu : r);
}
}  // namespace f16w

struct StF16W {
    using T = unsigned short;
    using R = float;
    static constexpr bool kShift = true;
    // the raw codec takes the population index; stores report saturation
    static constexpr bool kPerPop = true, kRange = true;
    template <int Q> static __device__ __forceinline__ float dec1(int n, unsigned h) { return f16w::decode<Q>(n, h); }
    template <int Q> static __device__ __forceinline__ float2 dec2(int n, unsigned w) {
        return make_float2(f16w::decode<Q>(n, w & 0xFFFFu), f16w::decode<Q>(n, w >> 16));
    }
    template <int Q> static __device__ __forceinline__ float ldr1(int n, const T* __restrict__ f, unsigned e) {
        return f16w::decode<Q>(n, __ldg(f + e));
    }
    template <int Q> static __device__ __forceinline__ float2 ldr2(int n, const T* __restrict__ f, unsigned e) {
        return dec2<Q>(n, __ldg(reinterpret_cast<const unsigned*>(f + e)));
    }
    template <int Q>
    static __device__ __forceinline__ void str1(int n, T* __restrict__ f, unsigned e, float v, unsigned& sat) {
        f[e] = (unsigned short)f16w::encode<Q>(n, v, sat);
    }
    template <int Q>
    static __device__ __forceinline__ void str2(int n, T* __restrict__ f, unsigned e, float2 v, unsigned& sat) {
        *reinterpret_cast<unsigned*>(f + e) = f16w::encode<Q>(n, v.x, sat) | (f16w::encode<Q>(n, v.y, sat) << 16);
    }
    // FP32 population f_n = w_n + g_n for the auxiliary kernels (moments,
    // sums, initialisation, host transfers); st_sat reports saturation (the
    // initialisation and upload kernels use it through st_chk).
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int n, unsigned e) {
        return ldr1<Q>(n, f, e) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int n, unsigned e, R v) {
        unsigned sat = 0;
        str1<Q>(n, f, e, v - (float)Lat<Q>::w(n), sat);
    }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return ldr1<Q>(n, f, (unsigned)(n * N + i)) + (float)Lat<Q>::w(n);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        unsigned sat = 0;
        f[n * N + i] = (unsigned short)f16w::encode<Q>(n, v - (float)Lat<Q>::w(n), sat);
    }
    template <int Q>
    static __device__ __forceinline__ void st_sat(T* __restrict__ f, int n, long long i, long long N, R v, unsigned& sat) {
        f[n * N + i] = (unsigned short)f16w::encode<Q>(n, v - (float)Lat<Q>::w(n), sat);
    }
    template <int Q> static __device__ __forceinline__ R rt(int n, R v) {
        unsigned sat = 0;
        return f16w::decode<Q>(n, f16w::encode<Q>(n, v - (float)Lat<Q>::w(n), sat)) + (float)Lat<Q>::w(n);
    }
};

// Raw loads and stores of the shifted value g_n of population n for any
// shifted policy (the per-population codec of StF16W takes n; the others
// ignore it), and the saturation report of the stores.
template <int Q, class St>
__device__ __forceinline__ float sh_ld1(int n, const typename St::T* __restrict__ f, unsigned e) {
    if constexpr (St::kPerPop) return St::template ldr1<Q>(n, f, e);
    else return St::ldr1(f, e);
}
template <int Q, class St>
__device__ __forceinline__ float2 sh_ld2(int n, const typename St::T* __restrict__ f, unsigned e) {
    if constexpr (St::kPerPop) return St::template ldr2<Q>(n, f, e);
    else return St::ldr2(f, e);
}
template <int Q, class St>
__device__ __forceinline__ void sh_st1(int n, typename St::T* __restrict__ f, unsigned e, float v, unsigned& sat) {
    if constexpr (St::kPerPop) St::template str1<Q>(n, f, e, v, sat);
    else St::str1(f, e, v);
}
template <int Q, class St>
__device__ __forceinline__ void sh_st2(int n, typename St::T* __restrict__ f, unsigned e, float2 v, unsigned& sat) {
    if constexpr (St::kPerPop) St::template str2<Q>(n, f, e, v, sat);
    else St::str2(f, e, v);
}
template <class St>
__device__ __forceinline__ void sh_report(const KParams& p, unsigned sat) {
    if constexpr (St::kRange) {
        if (sat > 0x7FFFu) atomicOr(p.flag, 4);
    }
}
// Store of population value v (compute type R) by the auxiliary kernels, with
// the saturation report of the policies whose stores can saturate; flag may
// be null (then saturation is not reported).
template <int Q, class St>
__device__ __forceinline__ void st_chk(typename St::T* __restrict__ f, int n, long long i, long long N,
                                       typename St::R v, unsigned& sat) {
    if constexpr (St::kRange) St::template st_sat<Q>(f, n, i, N, v, sat);
    else St::template st<Q>(f, n, i, N, v);
}
template <class St>
__device__ __forceinline__ void report_to(int* flag, unsigned sat) {
    if constexpr (St::kRange) {
        if (flag && sat > 0x7FFFu) atomicOr(flag, 4);
    }
}

// 64-bit fixed point (MPH_PREC_F64X): the stored integer is h_n = f_n / w_n
// in units of 2^-56.  Loads and stores convert to/from FP64 for the
// auxiliary kernels (moments, init, sums, host transfers); the step kernel of
// k_f64x.cu works on the integers directly.
constexpr int kFxShift = 56;
struct StF64X {
    using T = long long;
    static constexpr bool kShift = false;
    static constexpr bool kPerPop = false, kRange = false;
    using R = double;
    template <int Q> static __device__ __forceinline__ R lde(const T* __restrict__ f, int n, unsigned e) {
        return ((double)__ldg(f + e) * 0x1p-56) / Lat<Q>::iw(n);
    }
    template <int Q> static __device__ __forceinline__ void ste(T* __restrict__ f, int n, unsigned e, R v) {
        f[e] = __double2ll_rn(v * Lat<Q>::iw(n) * 0x1p56);
    }
    template <int Q> static __device__ __forceinline__ R ld(const T* __restrict__ f, int n, long long i, long long N) {
        return ((double)__ldg(f + n * N + i) * 0x1p-56) / Lat<Q>::iw(n);
    }
    template <int Q> static __device__ __forceinline__ void st(T* __restrict__ f, int n, long long i, long long N, R v) {
        f[n * N + i] = __double2ll_rn(v * Lat<Q>::iw(n) * 0x1p56);
    }
    template <int Q> static __device__ __forceinline__ R rt(int n, R v) {
        return ((double)__double2ll_rn(v * Lat<Q>::iw(n) * 0x1p56) * 0x1p-56) / Lat<Q>::iw(n);
    }
};

// ---------------------------------------------------------------------------
// Pull with link-wise boundary conditions.
// ---------------------------------------------------------------------------

// Value the reference's ghost fill stores at ghost g = x - c_n for population
// n, evaluated from the populations of x itself (the ghost-fill source cell
// g + c_n is x):
//   BounceBack family (BCTypes/BounceBack.H:36-63; NoSlip with rho=1, U=0,
//   NoSlipKernel.H:20-28; MovingWall, Inflow with the resolved rho, U):
//       f(x, opp n) + (((-2 rho) w_opp) (c_opp . U)) cs2inv
//   Outflow (OutflowKernel.H:26-38):           f(x, n)
//   PressureOutlet (PressureOutletKernel.H:29-64):
//       -f(x, opp n) + 2 w_n rho_out (1 + 0.5 cu^2 cs2inv^2 - 0.5 uu cs2inv)
// Rare path: reads its constants from the global copy pg of the parameters.
template <int Q, class St>
__device__ __noinline__ typename St::R boundary_value(const KParams* __restrict__ pg, int n, int cls,
                                                      const typename St::T* __restrict__ fin, long long c) {
    using L = Lat<Q>;
    using R = typename St::R;
    const long long N = pg->ncell;
    const int t = pg->bc_type[cls];
    const int o = L::opp(n);
    if (t == kBcOutflow) return St::template ld<Q>(fin, n, c, N);
    if (t == kBcPressure) {
        R rho = R(0.0), j0 = R(0.0), j1 = R(0.0), j2 = R(0.0);
#pragma unroll
        for (int m = 0; m < Q; ++m) {
            const R fm = St::template ld<Q>(fin, m, c, N);
            rho += fm;
            j0 += (R)L::cx(m) * fm;
            j1 += (R)L::cy(m) * fm;
            if (L::D == 3) j2 += (R)L::cz(m) * fm;
        }
        const R inv_rho = R(1.0) / rho;
        R cu, uu;
        if (L::D == 2) {
            cu = ((R)L::cx(n) * j0 + (R)L::cy(n) * j1) * inv_rho;
            uu = (j0 * j0 + j1 * j1) * inv_rho * inv_rho;
        } else {
            cu = ((R)L::cx(n) * j0 + (R)L::cy(n) * j1 + (R)L::cz(n) * j2) * inv_rho;
            uu = (j0 * j0 + j1 * j1 + j2 * j2) * inv_rho * inv_rho;
        }
        const R rho_out = (R)pg->bc_rho[cls];
        const R feq_even = (R)L::w(n) * rho_out *
                           (R(1.0) + R(0.5) * cu * cu * R(3.0) * R(3.0) - R(0.5) * uu * R(3.0));
        return -St::template ld<Q>(fin, o, c, N) + R(2.0) * feq_even;
    }
    if (t == kBcPeriodic) return R(__longlong_as_double(0x7ff8000000000000ULL));  // unreachable
    R rho = R(1), U0 = R(0.), U1 = R(0.), U2 = R(0.);
    if (t != kBcNoSlip) {
        rho = (R)pg->bc_rho[cls];
        U0 = (R)pg->bc_U[cls][0];
        U1 = (R)pg->bc_U[cls][1];
        U2 = (R)pg->bc_U[cls][2];
    }
    R cdotu;
    if (L::D == 2) cdotu = (R)L::cx(o) * U0 + (R)L::cy(o) * U1;
    else cdotu = (R)L::cx(o) * U0 + (R)L::cy(o) * U1 + (R)L::cz(o) * U2;
    const R contrib = R(-2.) * rho * (R)L::w(o) * cdotu * R(3.0);
    return St::template ld<Q>(fin, o, c, N) + contrib;
}

// Pull of a cell next to the domain boundary: periodic wrap, or the link-wise
// boundary value for ghosts outside a non-periodic face.
template <int Q, class St>
__device__ __forceinline__ void pull_edge(const KParams& p, const KParams* __restrict__ pg,
                                          const typename St::T* __restrict__ fin, int x, int y, int z, long long c,
                                          typename St::R* f) {
    using L = Lat<Q>;
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        int gx = x - L::cx(n), gy = y - L::cy(n), gz = z - L::cz(n);
        int k0 = 0, k1 = 0, k2 = 0;
        if (gx < 0) { if (p.periodic[0]) gx += p.nx; else k0 = -1; }
        else if (gx >= p.nx) { if (p.periodic[0]) gx -= p.nx; else k0 = 1; }
        if (gy < 0) { if (p.periodic[1]) gy += p.ny; else k1 = -1; }
        else if (gy >= p.ny) { if (p.periodic[1]) gy -= p.ny; else k1 = 1; }
        if (L::D == 3) {
            if (gz < 0) { if (p.periodic[2]) gz += p.nz; else k2 = -1; }
            else if (gz >= p.nz) { if (p.periodic[2]) gz -= p.nz; else k2 = 1; }
        }
        if ((k0 | k1 | k2) == 0) {
            const long long g = ((long long)gz * p.ny + gy) * p.nx + gx;
            // Obstacle link: bounce-back with U = 0 (BounceBack.H:36-63 at an
            // interior solid cell): the cell's own opposite population.
            if (p.cls && p.cls[g] == kSolid) f[n] = St::template ld<Q>(fin, L::opp(n), c, p.ncell);
            else f[n] = St::template ld<Q>(fin, n, g, p.ncell);
        } else {
            const int cls = (k0 + 1) + 3 * (k1 + 1) + (L::D == 3 ? 9 * (k2 + 1) : 0);
            f[n] = boundary_value<Q, St>(pg, n, cls, fin, c);
        }
    }
}

// Offsets (in cells) of the upstream neighbour along each axis, with the
// periodic wrap folded in: xm is the offset of x-1, xp of x+1, etc.  `wall`
// marks a cell next to a non-periodic face, which needs the boundary rules.
struct Nbr {
    int xm, xp, ym, yp, zm, zp;
    bool wall;
};

template <int D>
__device__ __forceinline__ Nbr neighbours(const KParams& p, int x, int y, int z) {
    Nbr o;
    const int nx = p.nx, ny = p.ny, nz = p.nz, plane = nx * ny;
    const bool x0 = x == 0, x1 = x == nx - 1, y0 = y == 0, y1 = y == ny - 1;
    o.xm = x0 ? nx - 1 : -1;
    o.xp = x1 ? -(nx - 1) : 1;
    o.ym = y0 ? (ny - 1) * nx : -nx;
    o.yp = y1 ? -(ny - 1) * nx : nx;
    o.wall = (!p.periodic[0] && (x0 || x1)) || (!p.periodic[1] && (y0 || y1));
    if (D == 3) {
        const bool z0 = z == 0, z1 = z == nz - 1;
        o.zm = z0 ? (nz - 1) * plane : -plane;
        o.zp = z1 ? -(nz - 1) * plane : plane;
        o.wall = o.wall || (!p.periodic[2] && (z0 || z1));
    } else {
        o.zm = o.zp = 0;
    }
    return o;
}

// Offset of the cell population n streams from: x - c_n.
template <int Q>
__device__ __forceinline__ int upstream(const Nbr& o, int n) {
    using L = Lat<Q>;
    const int ox = L::cx(n) == 1 ? o.xm : (L::cx(n) == -1 ? o.xp : 0);
    const int oy = L::cy(n) == 1 ? o.ym : (L::cy(n) == -1 ? o.yp : 0);
    const int oz = L::cz(n) == 1 ? o.zm : (L::cz(n) == -1 ? o.zp : 0);
    return ox + oy + oz;
}

// Pull through the wrapped neighbour offsets only, for callers that compute
// the cells next to non-periodic faces separately (the batch): every address
// stays inside the domain, and a wall cell's result is overwritten.
template <int Q, class St>
__device__ __forceinline__ void pull_interior(const KParams& p, const typename St::T* __restrict__ fin, int x, int y,
                                              int z, long long c, typename St::R* f) {
    using L = Lat<Q>;
    const Nbr o = neighbours<L::D>(p, x, y, z);
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
    for (int n = 0; n < Q; ++n)
        f[n] = St::template lde<Q>(fin, n, (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n)));
}
template <int Q, class St>
__device__ __forceinline__ void pull_shift_interior(const KParams& p, const typename St::T* __restrict__ fin, int x,
                                                    int y, int z, long long c, float* g) {
    using L = Lat<Q>;
    const Nbr o = neighbours<L::D>(p, x, y, z);
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
    for (int n = 0; n < Q; ++n) g[n] = sh_ld1<Q, St>(n, fin, (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n)));
}

// Pull of all Q populations into f.  Cells away from non-periodic faces use
// 32-bit element indices (Q * N < 2^32 is checked when a handle is created);
// cells next to a wall take pull_edge.
template <int Q, class St>
__device__ __forceinline__ void pull(const KParams& p, const KParams* __restrict__ pg,
                                     const typename St::T* __restrict__ fin, int x, int y, int z, long long c,
                                     typename St::R* f) {
    using L = Lat<Q>;
    const Nbr o = neighbours<L::D>(p, x, y, z);
    if (!o.wall && !(p.cls && p.cls[c] != kFluid)) {
        const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
        for (int n = 0; n < Q; ++n) {
            const unsigned e = (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n));
            f[n] = St::template lde<Q>(fin, n, e);
        }
    } else {
        pull_edge<Q, St>(p, pg, fin, x, y, z, c, f);
    }
}

// ---------------------------------------------------------------------------
// Moments and collision.
// ---------------------------------------------------------------------------

// rho = sum f and u = (sum c f [+ F/2]) / rho in the reference's order
// (Macroscopic.H:36-45, 158-204, 226-278).  Terms with c = 0 are skipped and
// c = -1 terms are subtracted: the running sums start at +0 and never become
// -0, so this is bit-identical to adding c*f.
template <int Q, bool FORCED>
__device__ __forceinline__ void moments_exact(const KParams& p, const double* f, double& rho, double* u) {
    using L = Lat<Q>;
    rho = 0.;
#pragma unroll
    for (int n = 0; n < Q; ++n) rho += f[n];
    double ux = 0., uy = 0., uz = 0.;
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        if (L::cx(n) == 1) ux += f[n];
        else if (L::cx(n) == -1) ux -= f[n];
        if (L::cy(n) == 1) uy += f[n];
        else if (L::cy(n) == -1) uy -= f[n];
        if (L::D == 3) {
            if (L::cz(n) == 1) uz += f[n];
            else if (L::cz(n) == -1) uz -= f[n];
        }
    }
    if (!FORCED) {
        u[0] = ux / rho;
        u[1] = uy / rho;
        u[2] = (L::D == 3) ? uz / rho : 0.0;
    } else {
        u[0] = (ux + p.hF[0]) / rho;
        u[1] = (uy + p.hF[1]) / rho;
        u[2] = (L::D == 3) ? (uz + p.hF[2]) / rho : 0.0;
    }
}

// c_n . u with the reference's left-to-right sum; zero components dropped
// (bit-identical: cu only enters through 1 + 3 cu, cu^2 and 3 cu * cF).
template <int Q, class R>
__device__ __forceinline__ R cdot(int n, const R* u) {
    using L = Lat<Q>;
    R s = R(0);
    bool first = true;
    const int c[3] = {L::cx(n), L::cy(n), L::cz(n)};
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
        if (c[d] == 0) continue;
        if (first) { s = (c[d] > 0) ? u[d] : -u[d]; first = false; }
        else s = (c[d] > 0) ? s + u[d] : s - u[d];
    }
    return s;
}

// Equilibrium (Equilibrium.H:28-57) + BGK (Collision.H:68-76) + Guo
// (Collision.H:21-65), reference operation order, in place on f.
template <int Q, bool FORCED>
__device__ __forceinline__ void collide_exact(const KParams& p, double* f) {
    using L = Lat<Q>;
    double rho, u[3];
    moments_exact<Q, FORCED>(p, f, rho, u);
    const double usq = (L::D == 2) ? u[0] * u[0] + u[1] * u[1] : u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double s = 1.5 * usq;  // 0.5 * cs2inv * u_sq
    double udotF = 0.0;
    if (FORCED) udotF = (L::D == 2) ? u[0] * p.F[0] + u[1] * p.F[1] : u[0] * p.F[0] + u[1] * p.F[1] + u[2] * p.F[2];
    const double omega = p.omega, omc = p.omc;
    {   // rest population: c = 0, so 1 + 3 cu + 4.5 cu^2 = 1 exactly
        const double feq = L::w(0) * rho * (1.0 - s);
        double o = omc * f[0] + omega * feq;
        if (FORCED) o = o + p.gpref[0] * ((p.gcF[0] + 0.0 * p.gcF[0]) - udotF);
        f[0] = o;
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const double cu = cdot<Q, double>(n, u);
        const double t3 = 3.0 * cu;
        const double sq = 4.5 * cu * cu;
        const double wr = L::w(n) * rho;
        const double feq_n = wr * (((1.0 + t3) + sq) - s);
        const double feq_m = wr * (((1.0 - t3) + sq) - s);
        double on = omc * f[n] + omega * feq_n;
        double om = omc * f[m] + omega * feq_m;
        if (FORCED) {
            on = on + p.gpref[n] * ((p.gcF[n] + t3 * p.gcF[n]) - udotF);
            om = om + p.gpref[m] * ((p.gcF[m] + (-t3) * p.gcF[m]) - udotF);
        }
        f[n] = on;
        f[m] = om;
    }
}

template <class R> __device__ __forceinline__ R recip(R x);
template <> __device__ __forceinline__ double recip<double>(double x) {
    // float reciprocal seed refined by two Newton steps: ~1 ulp.
    double r = (double)__frcp_rn((float)x);
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}
template <> __device__ __forceinline__ float recip<float>(float x) { return __frcp_rn(x); }

// Refactored BGK (+Guo) in compute type R, FMA-friendly:
//   out_n = f_n + omega (feq_n - f_n) [+ guo_n],
//   feq_{n, opp} = w rho (B + 4.5 cu^2 +- 3 cu),  B = 1 - 1.5 u^2.
template <int Q, class R, bool FORCED>
__device__ __forceinline__ void collide_fast(const KParams& p, R* f) {
    using L = Lat<Q>;
    using P = Prm<R>;
    R rho = f[0], jx = R(0), jy = R(0), jz = R(0);
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const R sm = f[n] + f[m];
        const R df = f[n] - f[m];
        rho += sm;
        if (L::cx(n) == 1) jx += df; else if (L::cx(n) == -1) jx -= df;
        if (L::cy(n) == 1) jy += df; else if (L::cy(n) == -1) jy -= df;
        if (L::D == 3) { if (L::cz(n) == 1) jz += df; else if (L::cz(n) == -1) jz -= df; }
    }
    const R inv = recip<R>(rho);
    R u[3];
    if (FORCED) {
        u[0] = (jx + P::hF(p, 0)) * inv;
        u[1] = (jy + P::hF(p, 1)) * inv;
        u[2] = (L::D == 3) ? (jz + P::hF(p, 2)) * inv : R(0);
    } else {
        u[0] = jx * inv;
        u[1] = jy * inv;
        u[2] = (L::D == 3) ? jz * inv : R(0);
    }
    const R usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const R B = R(1) - R(1.5) * usq;
    const R omega = P::omega(p);
    R udotF = R(0);
    if (FORCED) udotF = u[0] * P::F(p, 0) + u[1] * P::F(p, 1) + u[2] * P::F(p, 2);
    {
        const R feq = (R)L::w(0) * rho * B;
        R o = f[0] + omega * (feq - f[0]);
        if (FORCED) o -= P::gpref(p, 0) * udotF;
        f[0] = o;
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const R cu = cdot<Q, R>(n, u);
        const R a = (R(4.5) * cu) * cu + B;
        const R b = R(3) * cu;
        const R wr = (R)L::w(n) * rho;
        const R feq_n = wr * (a + b);
        const R feq_m = wr * (a - b);
        R on = f[n] + omega * (feq_n - f[n]);
        R om = f[m] + omega * (feq_m - f[m]);
        if (FORCED) {
            const R cF = P::gcF(p, n);
            on += P::gpref(p, n) * ((cF + b * cF) - udotF);
            om += P::gpref(p, m) * ((b * cF - cF) - udotF);
        }
        f[n] = on;
        f[m] = om;
    }
}


// ---------------------------------------------------------------------------
// Shifted FP32 collide for the 16-bit storage policies: the state is
// g_n = f_n - w_n, so rho = 1 + sum g and j = sum c g (sum w = 1, sum c w = 0),
// and the post-collision value is
//   g'_n = (1 - omega) g_n + omega (feq_n - w_n) [+ Guo term],
//   omega (feq_n - w_n) = (omega w_n rho) (3 c.u + 4.5 (c.u)^2 - 1.5 u.u)
//                         + omega w_n (rho - 1),
// one FMA per population after the per-pair terms.  The arithmetic is
// written with explicitly rounded operations over a value type V: float (one
// cell per thread) or float2 (two cells per thread, packed FP32x2
// instructions of sm_100 and later), so both forms round identically.
// ---------------------------------------------------------------------------
struct A1 {
    using V = float;
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ V splat(float c) { return c; }
    static __device__ __forceinline__ V rcp(V a) { return rcp_nr(a); }
    // 1/x for x near 1: hardware approximation refined by one Newton step.
    static __device__ __forceinline__ float rcp_nr(float x) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        const float e = __fmaf_rn(-x, r, 1.0f);
        return __fmaf_rn(r, e, r);
    }
};
struct A2 {
    using V = float2;
    static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
    static __device__ __forceinline__ V splat(float c) { return make_float2(c, c); }
    static __device__ __forceinline__ V rcp(V a) { return make_float2(A1::rcp_nr(a.x), A1::rcp_nr(a.y)); }
};

// acc (+/-)= v; `have` says whether acc holds a value yet (folded at compile
// time after unrolling).
template <class A>
__device__ __forceinline__ void acc_signed(typename A::V& acc, bool& have, int sign, typename A::V v) {
    if (sign == 0) return;
    const typename A::V m1 = A::splat(-1.0f);
    if (sign > 0) acc = have ? A::add(acc, v) : v;
    else acc = have ? A::fma(m1, v, acc) : A::mul(m1, v);
    have = true;
}

template <int Q, class A>
__device__ __forceinline__ typename A::V cdot_s(int n, const typename A::V* u) {
    using L = Lat<Q>;
    typename A::V r = A::splat(0.0f);
    bool have = false;
    acc_signed<A>(r, have, L::cx(n), u[0]);
    acc_signed<A>(r, have, L::cy(n), u[1]);
    if (L::D == 3) acc_signed<A>(r, have, L::cz(n), u[2]);
    return r;
}

template <int Q, class A, bool FORCED>
__device__ __forceinline__ void collide_shift(const KParams& p, typename A::V* g) {
    using L = Lat<Q>;
    using V = typename A::V;
    const V m1 = A::splat(-1.0f);
    V dr = g[0], j[3] = {A::splat(0.0f), A::splat(0.0f), A::splat(0.0f)};
    bool hj[3] = {false, false, false};
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const V sm = A::add(g[n], g[m]);
        const V df = A::fma(m1, g[m], g[n]);
        dr = A::add(dr, sm);
        acc_signed<A>(j[0], hj[0], L::cx(n), df);
        acc_signed<A>(j[1], hj[1], L::cy(n), df);
        if (L::D == 3) acc_signed<A>(j[2], hj[2], L::cz(n), df);
    }
    const V rho = A::add(A::splat(1.0f), dr);
    const V inv = A::rcp(rho);
    V u[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a == 2 && L::D == 2) { u[a] = A::splat(0.0f); continue; }
        u[a] = FORCED ? A::mul(A::add(j[a], A::splat(p.hF_f[a])), inv) : A::mul(j[a], inv);
    }
    V usq = A::mul(u[0], u[0]);
    usq = A::fma(u[1], u[1], usq);
    if (L::D == 3) usq = A::fma(u[2], u[2], usq);
    const V Bp = A::mul(A::splat(-1.5f), usq);
    const float om = p.omega_f;
    const V omc = A::splat(1.0f - om);
    V U = A::splat(0.0f);
    if (FORCED) {
        U = A::mul(u[0], A::splat(p.F_f[0]));
        U = A::fma(u[1], A::splat(p.F_f[1]), U);
        if (L::D == 3) U = A::fma(u[2], A::splat(p.F_f[2]), U);
    }
    {
        const float ow = om * (float)L::w(0);
        V e = A::fma(A::mul(A::splat(ow), rho), Bp, A::mul(A::splat(ow), dr));
        if (FORCED) e = A::fma(A::splat(-p.gpref_f[0]), U, e);
        g[0] = A::fma(omc, g[0], e);
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const float ow = om * (float)L::w(n);
        const V Ak = A::mul(A::splat(ow), rho);
        const V Ck = A::mul(A::splat(ow), dr);
        const V cu = cdot_s<Q, A>(n, u);
        const V b = A::mul(A::splat(3.0f), cu);
        const V ap = A::fma(A::mul(A::splat(4.5f), cu), cu, Bp);
        V en = A::fma(Ak, A::add(ap, b), Ck);
        V em = A::fma(Ak, A::fma(m1, b, ap), Ck);
        if (FORCED) {
            // Guo: gpref_n ((c_n.F)(1 + 3 c_n.u) - u.F); c_m = -c_n.
            const float qn = p.gpref_f[n] * p.gcF_f[n];
            const V nGU = A::mul(A::splat(-p.gpref_f[n]), U);
            en = A::add(en, A::fma(b, A::splat(qn), A::add(nGU, A::splat(qn))));
            em = A::add(em, A::fma(b, A::splat(qn), A::add(nGU, A::splat(-qn))));
        }
        g[n] = A::fma(omc, g[n], en);
        g[m] = A::fma(omc, g[m], em);
    }
}

// Pull of g = f - w for the shifted policies: raw values away from walls, the
// boundary rules (on f) next to them.
template <int Q, class St>
__device__ __forceinline__ void pull_shift(const KParams& p, const KParams* __restrict__ pg,
                                           const typename St::T* __restrict__ fin, int x, int y, int z, long long c,
                                           float* g) {
    using L = Lat<Q>;
    const Nbr o = neighbours<L::D>(p, x, y, z);
    if (!o.wall && !(p.cls && p.cls[c] != kFluid)) {
        const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
        for (int n = 0; n < Q; ++n) g[n] = sh_ld1<Q, St>(n, fin, (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n)));
    } else {
        pull_edge<Q, St>(p, pg, fin, x, y, z, c, g);
#pragma unroll
        for (int n = 0; n < Q; ++n) g[n] = __fadd_rn(g[n], -(float)L::w(n));
    }
}

// One step of one cell for any storage policy: pull, collide, store.
template <int Q, class St, int ARITH, bool FORCED>
__device__ __forceinline__ void step_cell(const KParams& p, const KParams* __restrict__ pg,
                                          const typename St::T* __restrict__ fin, typename St::T* __restrict__ fout,
                                          int x, int y, int z) {
    using R = typename St::R;
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
    if (p.cls && p.cls[c] == kSolid) {  // obstacle cell: rest state f = w
        unsigned sat = 0;
#pragma unroll
        for (int n = 0; n < Q; ++n) {
            if constexpr (St::kShift) sh_st1<Q, St>(n, fout, (unsigned)n * N + ci, 0.0f, sat);
            else St::template ste<Q>(fout, n, (unsigned)n * N + ci, (typename St::R)Lat<Q>::w(n));
        }
        return;
    }
    if constexpr (St::kShift) {
        float g[Q];
        pull_shift<Q, St>(p, pg, fin, x, y, z, c, g);
        collide_shift<Q, A1, FORCED>(p, g);
        unsigned sat = 0;
#pragma unroll
        for (int n = 0; n < Q; ++n) sh_st1<Q, St>(n, fout, (unsigned)n * N + ci, g[n], sat);
        sh_report<St>(p, sat);
    } else {
        R f[Q];
        pull<Q, St>(p, pg, fin, x, y, z, c, f);
        if constexpr (ARITH == kExact) collide_exact<Q, FORCED>(p, f);
        else collide_fast<Q, R, FORCED>(p, f);
#pragma unroll
        for (int n = 0; n < Q; ++n) St::template ste<Q>(fout, n, (unsigned)n * N + ci, f[n]);
    }
}

// ---------------------------------------------------------------------------
// Kernels on the handle's SoA state (no ghost layer).
// Block (BX, BY): lanes run along x so every warp shares (y, z).
// ---------------------------------------------------------------------------
template <int Q, class St, int ARITH, bool FORCED>
__global__ void __launch_bounds__(256) k_step(const typename St::T* __restrict__ fin, typename St::T* __restrict__ fout,
                                              const KParams p, const KParams* __restrict__ pg) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = p.y0 + blockIdx.y * blockDim.y + threadIdx.y;
    const int z = p.z0 + blockIdx.z;
    if (x >= p.nx || y >= p.y1) return;
    step_cell<Q, St, ARITH, FORCED>(p, pg, fin, fout, x, y, z);
}

// Shifted 16-bit policies with nx even: each thread advances the cell pair
// (x, x+1), x even, with packed FP32x2 arithmetic.  Populations with c_x = 0
// come from an aligned pair and are read as one 32-bit word; all stores are
// 32-bit words.  (nx even makes every row, plane and population offset even.)
// Registers sized for 3 blocks of 256 threads (80: 24 warps per SM); a
// 64-register build (32 warps, some spilling) measured 2 % slower.
template <int Q, class St, bool FORCED>
__global__ void __launch_bounds__(256, 3) k_step_pair(const typename St::T* __restrict__ fin,
                                                   typename St::T* __restrict__ fout, const KParams p,
                                                   const KParams* __restrict__ pg) {
    using L = Lat<Q>;
    const int x = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = p.y0 + blockIdx.y * blockDim.y + threadIdx.y;
    const int z = p.z0 + blockIdx.z;
    if (x >= p.nx || y >= p.y1) return;
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
    if (p.cls && (p.cls[c] | p.cls[c + 1]) != kFluid) {  // obstacle or its neighbour: one cell at a time
        step_cell<Q, St, kFast, FORCED>(p, pg, fin, fout, x, y, z);
        step_cell<Q, St, kFast, FORCED>(p, pg, fin, fout, x + 1, y, z);
        return;
    }
    const Nbr oa = neighbours<L::D>(p, x, y, z);
    // Cell b = x + 1 shares y, z with cell a, so its upstream offsets equal
    // a's except for the x wrap: c_x = +1 pulls from x, which for a at x = 0
    // wrapped by nx; c_x = -1 wraps by -nx for b at nx - 1.  When a is not
    // next to a face, b is next to one only if it is the last cell of a row
    // with non-periodic x faces.
    const bool b_xface = !p.periodic[0] && x + 2 == p.nx;
    const int dxm = x == 0 ? -p.nx : 0, dxp = x + 2 == p.nx ? -p.nx : 0;
    float2 g[Q];
    if (!oa.wall && !b_xface) {
#pragma unroll
        for (int n = 0; n < Q; ++n) {
            const unsigned ea = (unsigned)n * N + (unsigned)((int)ci + upstream<Q>(oa, n));
            if (L::cx(n) == 0) {
                g[n] = sh_ld2<Q, St>(n, fin, ea);
            } else {
                const unsigned eb = ea + 1u + (unsigned)(L::cx(n) == 1 ? dxm : dxp);
                g[n] = make_float2(sh_ld1<Q, St>(n, fin, ea), sh_ld1<Q, St>(n, fin, eb));
            }
        }
    } else {
        float ga[Q], gb[Q];
        pull_shift<Q, St>(p, pg, fin, x, y, z, c, ga);
        pull_shift<Q, St>(p, pg, fin, x + 1, y, z, c + 1, gb);
#pragma unroll
        for (int n = 0; n < Q; ++n) g[n] = make_float2(ga[n], gb[n]);
    }
    collide_shift<Q, A2, FORCED>(p, g);
    unsigned sat = 0;
#pragma unroll
    for (int n = 0; n < Q; ++n) sh_st2<Q, St>(n, fout, (unsigned)n * N + ci, g[n], sat);
    sh_report<St>(p, sat);
}

// updateMacroscopic (SimulationSetup.cpp:142-166): moments of the streamed
// populations, written as FP64 rho[c], u[d*N + c].
template <int Q, class St, bool FORCED>
__global__ void __launch_bounds__(256) k_moments(const typename St::T* __restrict__ fin, double* __restrict__ rho_out,
                                                 double* __restrict__ u_out, const KParams p,
                                                 const KParams* __restrict__ pg) {
    using R = typename St::R;
    using L = Lat<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= p.nx || y >= p.ny) return;
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    R fr[Q];
    pull<Q, St>(p, pg, fin, x, y, z, c, fr);
    double f[Q];
#pragma unroll
    for (int n = 0; n < Q; ++n) f[n] = (double)fr[n];
    double rho, u[3];
    moments_exact<Q, FORCED>(p, f, rho, u);
    rho_out[c] = rho;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u_out[d * p.ncell + c] = u[d];
}

// setInitialConditions (SimulationSetup.cpp:201-219): forced runs shift u by
// -F/(2 rho) (initVelCorrection, Macroscopic.cpp:164-181), f = feq(rho, u)
// (computeEquilibrium, Equilibrium.cpp:32-43), and the macroscopic fields are
// recomputed from the stored f (computeMacroscopic, Macroscopic.cpp:139-162).
template <int Q, class St, bool FORCED>
__global__ void __launch_bounds__(256) k_init(typename St::T* __restrict__ fout, double* __restrict__ rho_io,
                                              double* __restrict__ u_io, const KParams p) {
    using L = Lat<Q>;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.ncell) return;
    const double rho = rho_io[c];
    double u[3] = {u_io[c], u_io[p.ncell + c], L::D == 3 ? u_io[2 * p.ncell + c] : 0.0};
    if (FORCED)
        for (int d = 0; d < L::D; ++d) u[d] = u[d] - 0.5 * p.F[d] / rho;
    const double usq = (L::D == 2) ? u[0] * u[0] + u[1] * u[1] : u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    double f[Q];
    unsigned sat = 0;
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const double cu = (n == 0) ? 0.0 : cdot<Q, double>(n, u);
        f[n] = L::w(n) * rho * (1 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        st_chk<Q, St>(fout, n, c, p.ncell, (typename St::R)f[n], sat);
    }
    report_to<St>(p.flag, sat);
    if (FORCED) {
        // moments of the stored values (as a reload would return them; the
        // read-only cache path must not re-read memory this kernel wrote)
        double fs[Q];
#pragma unroll
        for (int n = 0; n < Q; ++n) fs[n] = (double)St::template rt<Q>(n, (typename St::R)f[n]);
        double r, uu[3];
        moments_exact<Q, true>(p, fs, r, uu);
        rho_io[c] = r;
        for (int d = 0; d < L::D; ++d) u_io[d * p.ncell + c] = uu[d];
    }
}

// Warm start (no counterpart in the reference): f = feq(rho, u) + f_neq with
// the first-order Chapman-Enskog non-equilibrium part of BGK.  The stored
// populations are post-collision (the next step's pull streams them), and a
// BGK collision scales the pre-collision part -(tau w rho / cs2) Q : grad u
// by (1 - omega), so
//   f_neq_n = -((tau - 1) w_n rho / cs2) (c_n c_n - cs2 I) : grad u,  cs2 = 1/3,
// grad u by central differences, one-sided where a neighbour lies beyond a
// non-periodic face or in an obstacle, zero with no fluid neighbour along an
// axis.  Obstacle cells get the rest state.  Unforced domains.
template <int Q, class St>
__global__ void __launch_bounds__(256) k_init_neq(typename St::T* __restrict__ fout, const double* __restrict__ rho_in,
                                                  const double* __restrict__ u_in, const KParams p) {
    using L = Lat<Q>;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.ncell) return;
    const long long N = p.ncell;
    if (p.cls && p.cls[c] == kSolid) {
#pragma unroll
        for (int n = 0; n < Q; ++n) St::template st<Q>(fout, n, c, N, (typename St::R)L::w(n));
        return;
    }
    const int x = (int)(c % p.nx), y = (int)((c / p.nx) % p.ny), z = (int)(c / ((long long)p.nx * p.ny));
    const double rho = rho_in[c];
    double u[3] = {u_in[c], u_in[N + c], L::D == 3 ? u_in[2 * N + c] : 0.0};
    double G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // G[a][b] = d_a u_b
    const int pos[3] = {x, y, z}, dims[3] = {p.nx, p.ny, p.nz};
    const long long stride[3] = {1, p.nx, (long long)p.nx * p.ny};
    for (int a = 0; a < L::D; ++a) {
        long long nb[2];
        bool ok[2];
        for (int s = 0; s < 2; ++s) {
            int q = pos[a] + (s ? 1 : -1);
            ok[s] = true;
            if (q < 0 || q >= dims[a]) {
                if (p.periodic[a]) q = q < 0 ? q + dims[a] : q - dims[a];
                else ok[s] = false;
            }
            nb[s] = c + (long long)(q - pos[a]) * stride[a];
            if (ok[s] && p.cls && p.cls[nb[s]] == kSolid) ok[s] = false;
        }
        for (int b = 0; b < L::D; ++b) {
            const double um = ok[0] ? u_in[b * N + nb[0]] : 0.0, up = ok[1] ? u_in[b * N + nb[1]] : 0.0;
            if (ok[0] && ok[1]) G[a][b] = 0.5 * (up - um);
            else if (ok[1]) G[a][b] = up - u[b];
            else if (ok[0]) G[a][b] = u[b] - um;
        }
    }
    const double tau = 1.0 / p.omega;
    const double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double divu = G[0][0] + G[1][1] + G[2][2];
    unsigned sat = 0;
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const double cu = cdot<Q, double>(n, u);
        const double feq = L::w(n) * rho * (1 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq);
        const int cv[3] = {L::cx(n), L::cy(n), L::cz(n)};
        double cc = 0.0;
        for (int a = 0; a < L::D; ++a)
            for (int b = 0; b < L::D; ++b) cc += cv[a] * cv[b] * G[a][b];
        const double neq = -3.0 * (tau - 1.0) * L::w(n) * rho * (cc - divu / 3.0);
        st_chk<Q, St>(fout, n, c, N, (typename St::R)(feq + neq), sat);
    }
    report_to<St>(p.flag, sat);
}

// FP64 sums of the stored populations: block partials (mass, jx, jy, jz)
// into part[4*block]; k_reduce_final adds them in block order.
template <int Q, class St>
__global__ void __launch_bounds__(256) k_reduce_partial(const typename St::T* __restrict__ fin, double* __restrict__ part,
                                                        long long ncell) {
    using L = Lat<Q>;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int n = 0; n < Q; ++n) {
            const double v = (double)St::template ld<Q>(fin, n, c, ncell);
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

}  // namespace mph
