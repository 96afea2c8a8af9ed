// fx_kernels.cuh -- device code of the FP64-accurate fixed-point step
// (MPH_PREC_F64X), shared by the single-domain kernels (k_f64x.cu) and the
// batch kernels (k_f64x_batch.cu).  The arithmetic and its range are
// described at the top of k_f64x.cu.
#pragma once

#include "lbm_kernels.cuh"

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

}  // namespace

}  // namespace mph
