// k_f64x.cu -- the FP64-accurate step on GB300's integer pipes.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (2 DFMA per SM per clock), so
// a D3Q19 cell update with ~170 FP64 operations is FP64-bound at ~15% of the
// HBM roofline.  This kernel keeps each population as a 64-bit fixed-point
// number h_n = f_n / w_n (resolution 2^-56 of a quantity of order one, far
// finer than FP64's 2^-53 relative rounding) and does the BGK+Guo update with
// integer adds and 64x64->high-64 multiplies (IMAD pipe):
//
//   rho = sum_k w_k S_k,  J = sum_k w_k (sum_{n in k} c_n h_n) + F/2
//   r = 1/rho (FP32 seed + two fixed-point Newton steps), u = J r
//   Pi = J u  (= rho u u),  A = rho - 1.5 tr(Pi)
//   feq_n / w_n = A + 3 c_n.J + 4.5 c_n c_n : Pi              (adds only)
//   guo_n / w_n = c_n.F' + 3 (c_n.u)(c_n.F') - u.F',  F' = 3 (1 - omega/2) F
//   h_n' = h_n + omega (feq_n/w_n - h_n) + guo_n/w_n          (1 multiply)
//
// which is the reference's BGK + Guo update (Collision.cpp:55-92,
// Collision.H:21-76, Equilibrium.H:43-57) in exact arithmetic; the rounding
// of the reference's FP64 evaluation (~1e-16 per operation) is the only
// difference, so results agree to ~1e-16 per step.  The HBM traffic is the
// same 2*Q*8 bytes per cell update as FP64 storage.
//
// Range: class sums of h within +-128, rho in (1/16, 64), |J|, |u| < 4 and
// |feq/w - h| < 32; a cell outside sets the handle's error flag (reported as
// MPH_ERR_NONFINITE by the host) instead of producing silent wrap-around.
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "lbm_launch.h"

namespace mph {

namespace {

using i64 = long long;
using u64 = unsigned long long;

// floor(a * b / 2^64) for signed a and unsigned b.
__device__ __forceinline__ i64 mulhi_su(i64 a, u64 b) {
    const u64 h = __umul64hi((u64)a, b);
    return (i64)(h - (a < 0 ? b : 0ull));
}
// floor(a * b / 2^64), both signed.
__device__ __forceinline__ i64 mulhi_ss(i64 a, i64 b) { return __mul64hi(a, b); }

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Value of the ghost population at g = x - c_n for cells next to a
// non-periodic face, in the fixed-point representation (see
// boundary_value in lbm_kernels.cuh for the rules and their reference).
template <int Q>
__device__ __noinline__ i64 boundary_value_x(const KParams* __restrict__ pg, const i64* __restrict__ kbb, int n,
                                             int cls, const i64* __restrict__ fin, long long c) {
    using L = Lat<Q>;
    const long long N = pg->ncell;
    const int t = pg->bc_type[cls];
    const int o = L::opp(n);
    if (t == kBcOutflow) return fin[n * N + c];
    if (t == kBcPressure) {
        const double v = boundary_value<Q, StF64X>(pg, n, cls, fin, c);
        return __double2ll_rn(v * L::iw(n) * 0x1p56);
    }
    // bounce-back family: h(x, opp n) + contrib / w_n, the constant folded on
    // the host from the reference's contrib (BCTypes/BounceBack.H:56-63).
    return fin[o * N + c] + kbb[cls * 27 + n];
}

template <int Q, bool OBST>
__device__ __forceinline__ void pull_x(const KParams& p, const KParams* __restrict__ pg, const i64* __restrict__ kbb,
                                       const i64* __restrict__ fin, int x, int y, int z, long long c, i64* h) {
    using L = Lat<Q>;
    const Nbr o = neighbours<L::D>(p, x, y, z);
    if (!o.wall && !(OBST && p.cls[c] != kFluid)) {
        const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
        for (int n = 0; n < Q; ++n) h[n] = __ldg(fin + ((unsigned)n * N + (unsigned)((int)ci + upstream<Q>(o, n))));
        return;
    }
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
            // Obstacle link: bounce-back with U = 0; w_opp = w_n, so in h = f / w
            // it is the cell's own opposite value.
            if (OBST && p.cls[g] == kSolid) h[n] = __ldg(fin + L::opp(n) * p.ncell + c);
            else h[n] = __ldg(fin + n * p.ncell + g);
        } else {
            const int cls = (k0 + 1) + 3 * (k1 + 1) + (L::D == 3 ? 9 * (k2 + 1) : 0);
            h[n] = boundary_value_x<Q>(pg, kbb, n, cls, fin, c);
        }
    }
}

// Products are formed with one or two extra fraction bits and rounded by
// (t + 1) >> 1 or (t + 2) >> 2: the 64x64 high-half multiply truncates, and a
// truncation bias would accumulate in the conserved mass over many steps,
// while rounded errors stay unbiased like the reference's FP64 rounding.
__device__ __forceinline__ i64 rnd1(i64 t) { return (t + 1) >> 1; }
__device__ __forceinline__ i64 rnd2(i64 t) { return (t + 2) >> 2; }
__device__ __forceinline__ i64 rnd4(i64 t) { return (t + 8) >> 4; }

// omega * d in Q.56, rounded to nearest.  W = omega/2 in Q0.64 with its low
// bit clear, wh1 = W/2 - 1.  With the sign bit of 4d flipped the operand is
// 4d + 2^63 >= 0, so one unsigned high multiply gives
// floor(4 d W / 2^64) + W/2 = floor(2 omega d) + W/2 (omega d with one extra
// fraction bit plus a known integer), and (t - wh1) >> 1 rounds it.
__device__ __forceinline__ i64 omega_mul(i64 d, u64 W, u64 wh1) {
    const u64 t = __umul64hi((u64)(d << 2) ^ (1ull << 63), W);
    return (i64)(t - wh1) >> 1;
}

// Weight of class k (|c|^2 = k) as a multiple of the smallest weight of the
// lattice: every lattice's weights are integer multiples of its smallest.
template <int Q>
__device__ __forceinline__ constexpr int wratio(int k) {
    return Q == 9 ? (k == 0 ? 16 : k == 1 ? 4 : 1)
         : Q == 15 ? (k == 0 ? 16 : k == 1 ? 8 : 1)
         : Q == 19 ? (k == 0 ? 12 : k == 1 ? 2 : 1)
                   : (k == 0 ? 64 : k == 1 ? 16 : k == 2 ? 4 : 1);
}

template <int Q, bool FORCED>
__device__ __forceinline__ void collide_x(const KParamsX& px, i64* h, int& bad) {
    using L = Lat<Q>;
    constexpr int D = L::D;
    constexpr bool has[4] = {true, true, Q == 9 || Q == 19 || Q == 27, Q == 15 || Q == 27};
    // Class sums of h and of c_a h (exact integer arithmetic).
    i64 sr[4] = {0, 0, 0, 0};
    i64 sj[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int n = 0; n < Q; ++n) {
        const int k = wclass<Q>(n);
        sr[k] += h[n];
        const int c[3] = {L::cx(n), L::cy(n), L::cz(n)};
#pragma unroll
        for (int a = 0; a < D; ++a) {
            if (c[a] == 1) sj[k][a] += h[n];
            else if (c[a] == -1) sj[k][a] -= h[n];
        }
    }
    // rho = w_min sum_k r_k S_k and J_a = w_min sum_k r_k T_ka (+ F_a/2):
    // the weighted sums are formed in Q.52 (headroom for r_k up to 64) and
    // multiplied once by Wm = 32 w_min (Q0.64) -> Q.57, rounded to Q.56.
    i64 rq = 0, jq[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!has[k]) continue;
        rq += wratio<Q>(k) * rnd4(sr[k]);
#pragma unroll
        for (int a = 0; a < D; ++a)
            if (k > 0) jq[a] += wratio<Q>(k) * rnd4(sj[k][a]);
    }
    const i64 rho = rnd1(mulhi_su(rq, px.Wm));
    i64 J[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
        J[a] = rnd1(mulhi_su(jq[a], px.Wm));
        if (FORCED) J[a] += px.hF[a];
    }
    // r = 1/rho in Q.60: FP32 seed (~2^-22) and one Newton step (~2^-44);
    // u only enters through Pi = J u and the force terms, where this
    // precision contributes < 1e-19 absolute.
    const float rf = (float)(int)(rho >> 32) * 0x1p-24f;
    u64 R = (u64)(unsigned)(rcp_approx(rf) * 0x1p27f) << 33;
    {
        const u64 P = __umul64hi((u64)rho, R);          // rho r in Q.52
        const i64 e = (i64)((1ull << 52) - P);           // 1 - rho r in Q.52
        R += (u64)(mulhi_su(e << 11, R) << 1);           // r e in Q.60
    }
    // u = J r and Pi = J u, Q.56.
    i64 J5[3] = {0, 0, 0}, u5[3] = {0, 0, 0}, u[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
        J5[a] = J[a] << 5;
        u[a] = rnd1(mulhi_su(J5[a], R));
        u5[a] = u[a] << 5;
    }
    i64 Pd[3] = {0, 0, 0}, Po[3] = {0, 0, 0};  // diagonal; off-diagonal (xy, xz, yz)
#pragma unroll
    for (int a = 0; a < D; ++a) Pd[a] = rnd2(mulhi_ss(J5[a], u5[a]));
    Po[0] = rnd2(mulhi_ss(J5[0], u5[1]));
    if (D == 3) {
        Po[1] = rnd2(mulhi_ss(J5[0], u5[2]));
        Po[2] = rnd2(mulhi_ss(J5[1], u5[2]));
    }
    {
        // range guard of the shifts above: rho in (1/16, 64), |J|, |u| < 4
        const u64 lim = 4ull << kFxShift;
        bool ok = rho > (1ll << (kFxShift - 4)) && rho < (64ll << kFxShift);
#pragma unroll
        for (int a = 0; a < D; ++a) ok = ok && (u64)(J[a] + (i64)lim) < 2 * lim && (u64)(u[a] + (i64)lim) < 2 * lim;
        bad |= !ok;
    }
    // Equilibrium moments in h-space: feq/w = A + c.J3 + sum_a c_a^2 P45_a
    // + sum_{a<b} c_a c_b P9_ab.
    const i64 tr = Pd[0] + Pd[1] + Pd[2];
    i64 A = rho - (tr + rnd1(tr));
    i64 J3[3], P45[3], P9[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        J3[a] = J[a] + (J[a] << 1);
        P45[a] = (Pd[a] << 2) + rnd1(Pd[a]);
        P9[a] = (Po[a] << 3) + Po[a];
    }
    if (FORCED) {
        // The Guo term divided by omega joins the same moments, so that
        // h' = h + omega (feq/w + guo/(w omega) - h) needs no extra work per
        // population: guo/(w omega) = c.Fw + 3 (c.u)(c.Fw) - u.Fw with
        // Fw = 3 (1 - omega/2) F / omega.
        i64 V[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int b = 0; b < D; ++b) {
            if (!(px.fmask & (1 << b))) continue;
#pragma unroll
            for (int a = 0; a < D; ++a) V[a][b] = rnd2(mulhi_ss(u5[a], px.Fw[b] << 5));
        }
        i64 uF = 0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            uF += V[a][a];
            P45[a] += 3 * V[a][a];
            J3[a] += px.Fw[a];
        }
        A -= uF;
        P9[0] += 3 * (V[0][1] + V[1][0]);
        if (D == 3) {
            P9[1] += 3 * (V[0][2] + V[2][0]);
            P9[2] += 3 * (V[1][2] + V[2][1]);
        }
    }
    // Bases shared by the populations of one face / edge / corner family.
    i64 Fb[3], Eb[3], Cb = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) Fb[a] = A + P45[a];
    Eb[0] = Fb[0] + P45[1];
    Eb[1] = Fb[0] + P45[2];
    Eb[2] = Fb[1] + P45[2];
    if (Q == 15 || Q == 27) Cb = Eb[0] + P45[2];

    const u64 W = px.W, wh1 = px.wh1;
    int dmag = 0;  // |d| < 32 for every population (high words within 2^29)
    {
        const i64 d = A - h[0];
        const int hi = (int)(d >> 32);
        dmag |= hi ^ (hi >> 31);
        h[0] += omega_mul(d, W, wh1);
    }
#pragma unroll
    for (int n = 1; n < Q; ++n) {
        const int m = L::opp(n);
        if (m < n) continue;
        const int c[3] = {L::cx(n), L::cy(n), L::cz(n)};
        const int nz = (c[0] != 0) + (c[1] != 0) + (c[2] != 0);
        i64 E, O = 0;
        if (nz == 1) {
            E = c[0] ? Fb[0] : (c[1] ? Fb[1] : Fb[2]);
        } else if (nz == 2) {
            const int k = c[0] == 0 ? 2 : (c[1] == 0 ? 1 : 0);
            const int sg = c[0] ? (c[1] ? c[0] * c[1] : c[0] * c[2]) : c[1] * c[2];
            E = (sg > 0) ? Eb[k] + P9[k] : Eb[k] - P9[k];
        } else {
            E = Cb;
            E += (c[0] * c[1] > 0) ? P9[0] : -P9[0];
            E += (c[0] * c[2] > 0) ? P9[1] : -P9[1];
            E += (c[1] * c[2] > 0) ? P9[2] : -P9[2];
        }
        bool first = true;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            if (c[a] == 0) continue;
            if (first) { O = (c[a] > 0) ? J3[a] : -J3[a]; first = false; }
            else O = (c[a] > 0) ? O + J3[a] : O - J3[a];
        }
        const i64 dn = (E + O) - h[n];
        const i64 dm = (E - O) - h[m];
        const int hn = (int)(dn >> 32), hm = (int)(dm >> 32);
        dmag |= (hn ^ (hn >> 31)) | (hm ^ (hm >> 31));
        h[n] += omega_mul(dn, W, wh1);
        h[m] += omega_mul(dm, W, wh1);
    }
    bad |= dmag >= (1 << 29);
}

// OBST: the domain has obstacles (p.cls set); the plain instantiation
// carries no class-byte test.  Launched in blocks of 128 threads along x
// (104 registers: 4 blocks, 16 warps per SM): 18.3 GLUPS at 512^3 against
// 17.9 for blocks of 256 with the same occupancy; capping the registers at
// 96 for 20 warps per SM measured 17.7.
// WIN: the launch covers the window (y0, y1, z0, z1) of p rather than the
// whole domain (the offsets cost about 1 % at 512^3 when always applied).
template <int Q, bool FORCED, bool OBST, bool WIN>
__global__ void __launch_bounds__(256) k_step_x(const i64* __restrict__ fin, i64* __restrict__ fout, const KParams p,
                                                const KParamsX px, const KParams* __restrict__ pg,
                                                const i64* __restrict__ kbb, int* __restrict__ flag) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = (WIN ? p.y0 : 0) + blockIdx.y * blockDim.y + threadIdx.y;
    const int z = (WIN ? p.z0 : 0) + blockIdx.z;
    if (x >= p.nx || y >= (WIN ? p.y1 : p.ny)) return;
    const long long c = ((long long)z * p.ny + y) * p.nx + x;
    const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
    if (OBST && p.cls[c] == kSolid) {  // obstacle cell: rest state, h = f / w = 1
#pragma unroll
        for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = 1LL << 56;
        return;
    }
    i64 h[Q];
    pull_x<Q, OBST>(p, pg, kbb, fin, x, y, z, c, h);
    int bad = 0;
    collide_x<Q, FORCED>(px, h, bad);
    if (bad) atomicOr(flag, 1);
#pragma unroll
    for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = h[n];
}

// Persistent, software-pipelined variant.  A tile is 256 consecutive cells of
// one row (y, z); each CTA walks the tiles with a grid stride.  Before the
// collide of tile t every thread issues cp.async copies of the Q values its
// cell of tile t + gridDim.x will pull into the other shared-memory stage, so
// the HBM latency of the next tile overlaps the integer arithmetic of this
// one without extra warps.  Each thread only reads what it copied itself, so
// the per-thread cp.async.wait_group is the only synchronisation.  Cells next
// to a non-periodic face (and lanes past the row end) skip the staging and
// use the direct boundary pull.
constexpr int kPipeThreads = 256;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

template <int Q>
__device__ __forceinline__ void tile_cell(const KParams& p, int tiles_per_row, int tile, int& x, int& y, int& z) {
    const int row = tile / tiles_per_row;
    x = (tile - row * tiles_per_row) * kPipeThreads + threadIdx.x;
    y = row % p.ny;
    z = row / p.ny;
}

template <int Q>
__device__ __forceinline__ void stage_tile(const KParams& p, const i64* __restrict__ fin, int tiles_per_row, int tile,
                                           i64* __restrict__ buf) {
    using L = Lat<Q>;
    int x, y, z;
    tile_cell<Q>(p, tiles_per_row, tile, x, y, z);
    if (x < p.nx) {
        const Nbr o = neighbours<L::D>(p, x, y, z);
        if (!o.wall) {
            const unsigned N = (unsigned)p.ncell;
            const int ci = (z * p.ny + y) * p.nx + x;
#pragma unroll
            for (int n = 0; n < Q; ++n)
                cp_async8(buf + n * kPipeThreads + threadIdx.x, fin + ((unsigned)n * N + (unsigned)(ci + upstream<Q>(o, n))));
        }
    }
    cp_async_commit();
}

template <int Q, bool FORCED>
__global__ void __launch_bounds__(kPipeThreads) k_step_x_pipe(const i64* __restrict__ fin, i64* __restrict__ fout,
                                                              const KParams p, const KParamsX px,
                                                              const KParams* __restrict__ pg,
                                                              const i64* __restrict__ kbb, int* __restrict__ flag,
                                                              int tiles_per_row, int ntiles) {
    using L = Lat<Q>;
    extern __shared__ i64 smem[];  // [2][Q][kPipeThreads]
    int stage = 0;
    int tile = blockIdx.x;
    if (tile < ntiles) stage_tile<Q>(p, fin, tiles_per_row, tile, smem);
    int bad = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        const int next = tile + gridDim.x;
        if (next < ntiles) stage_tile<Q>(p, fin, tiles_per_row, next, smem + (stage ^ 1) * Q * kPipeThreads);
        else cp_async_commit();
        cp_async_wait1();
        int x, y, z;
        tile_cell<Q>(p, tiles_per_row, tile, x, y, z);
        if (x < p.nx) {
            const long long c = ((long long)z * p.ny + y) * p.nx + x;
            const Nbr o = neighbours<L::D>(p, x, y, z);
            i64 h[Q];
            if (!o.wall) {
                const i64* b = smem + stage * Q * kPipeThreads + threadIdx.x;
#pragma unroll
                for (int n = 0; n < Q; ++n) h[n] = b[n * kPipeThreads];
            } else {
                pull_x<Q, false>(p, pg, kbb, fin, x, y, z, c, h);
            }
            collide_x<Q, FORCED>(px, h, bad);
            const unsigned N = (unsigned)p.ncell, ci = (unsigned)c;
#pragma unroll
            for (int n = 0; n < Q; ++n) fout[(unsigned)n * N + ci] = h[n];
        }
        stage ^= 1;
    }
    if (bad) atomicOr(flag, 1);
}

}  // namespace

namespace {
template <int Q, bool FORCED, bool OBST, bool WIN>
void step_x_launch(const i64* fin, i64* fout, const KParams& p, const KParamsX& px, const KParams* pg, const i64* kbb,
                   int* flag, cudaStream_t s) {
    dim3 g, b;
    step_shape(p, g, b, 128);
    if (const char* env = std::getenv("MPH_F64X_BLOCK")) {  // "BXxBY": other block shapes
        int bx = 0, by = 0;
        if (std::sscanf(env, "%dx%d", &bx, &by) == 2 && bx >= 32 && bx % 32 == 0 && by >= 1 && bx * by <= 256) {
            b = dim3(bx, by, 1);
            g = dim3((p.nx + bx - 1) / bx, (p.y1 - p.y0 + by - 1) / by, p.z1 - p.z0);
        }
    }
    k_step_x<Q, FORCED, OBST, WIN><<<g, b, 0, s>>>(fin, fout, p, px, pg, kbb, flag);
}

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

// Three run-time flags to compile-time constants.
template <class F>
cudaError_t with_flags(bool a, bool b, bool c, F&& f) {
    using T = std::true_type;
    using N = std::false_type;
    if (a) {
        if (b) return c ? f(T{}, T{}, T{}) : f(T{}, T{}, N{});
        return c ? f(T{}, N{}, T{}) : f(T{}, N{}, N{});
    }
    if (b) return c ? f(N{}, T{}, T{}) : f(N{}, T{}, N{});
    return c ? f(N{}, N{}, T{}) : f(N{}, N{}, N{});
}

template <int Q, bool FORCED>
cudaError_t pipe_setup(size_t& smem) {
    smem = 2 * Q * kPipeThreads * sizeof(long long);
    return cudaFuncSetAttribute(k_step_x_pipe<Q, FORCED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
}  // namespace

int f64x_pipe_ctas(int q, bool forced) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    size_t smem = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define MPH_XP_OCC(QQ)                                                                                         \
    case QQ:                                                                                                   \
        e = forced ? pipe_setup<QQ, true>(smem) : pipe_setup<QQ, false>(smem);                                 \
        if (e == cudaSuccess)                                                                                  \
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                                 \
                &per_sm, forced ? k_step_x_pipe<QQ, true> : k_step_x_pipe<QQ, false>, kPipeThreads, smem);    \
        break;
    switch (q) {
        MPH_XP_OCC(9)
        MPH_XP_OCC(15)
        MPH_XP_OCC(19)
        MPH_XP_OCC(27)
    }
#undef MPH_XP_OCC
    if (e != cudaSuccess) return 0;
    return per_sm * sms;
}

cudaError_t launch_step_f64x_pipe(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                                  const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                                  int ctas, cudaStream_t s) {
    const int tiles_per_row = (p.nx + kPipeThreads - 1) / kPipeThreads;
    const int ntiles = tiles_per_row * p.ny * p.nz;
    const int grid = ctas < ntiles ? ctas : ntiles;
    const size_t sm = 2 * (size_t)q * kPipeThreads * sizeof(long long);
#define MPH_XP_CASE(QQ)                                                                                       \
    case QQ:                                                                                                  \
        if (forced)                                                                                           \
            k_step_x_pipe<QQ, true><<<grid, kPipeThreads, sm, s>>>(fin, fout, p, px, pg, kbb, flag, tiles_per_row, ntiles);  \
        else                                                                                                  \
            k_step_x_pipe<QQ, false><<<grid, kPipeThreads, sm, s>>>(fin, fout, p, px, pg, kbb, flag, tiles_per_row, ntiles); \
        return cudaGetLastError();
    switch (q) {
        MPH_XP_CASE(9)
        MPH_XP_CASE(15)
        MPH_XP_CASE(19)
        MPH_XP_CASE(27)
    }
#undef MPH_XP_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_step_f64x(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                             const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                             cudaStream_t s) {
    const bool win = p.y0 != 0 || p.y1 != p.ny || p.z0 != 0 || p.z1 != p.nz;
    return with_q(q, [&](auto qc) {
        constexpr int Q = decltype(qc)::value;
        return with_flags(forced, p.cls != nullptr, win, [&](auto fc, auto oc, auto wc) {
            step_x_launch<Q, decltype(fc)::value, decltype(oc)::value, decltype(wc)::value>(fin, fout, p, px, pg,
                                                                                            kbb, flag, s);
            return cudaGetLastError();
        });
    });
}

}  // namespace mph
