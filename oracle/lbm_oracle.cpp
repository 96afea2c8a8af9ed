// lbm_oracle.cpp -- CPU oracle for the lattice-Boltzmann time step.
//
// TEST INFRASTRUCTURE ONLY: the checker that the CUDA product is compared
// against (tests/, __graft_entry__.smoke(), bench.py's CPU baseline arm).  The
// product library never links or calls it.
//
// It restates the reference's CPU path with the reference's data structure
// (one ghost-grown FAB per population set, FillBoundary then the physical BC
// ghost fill) and with the reference's floating-point operation order, so that
// results are bit-identical to the reference when built with
// -ffp-contract=off.  Each routine cites the reference file:line it follows
// (paths relative to the reference project root).  Its parity is pinned by
// tests/golden/ fixtures produced by the reference's own LBM sources compiled
// under oracle/_ref/ (see oracle/build_ref.sh and tests/golden/make_golden.py).
#include "oracle_api.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { BC_MOVING = 0, BC_NOSLIP = 1, BC_INFLOW = 2, BC_OUTFLOW = 3, BC_PRESSURE = 4, BC_PERIODIC = 5 };

// Velocity sets, q ordering and weights of src/LBM/LatticeDescriptor.H:23-263.
template <int D, int Q> struct Lat;
template <> struct Lat<2, 9> {
    static constexpr int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    static constexpr int cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    static constexpr int cz[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    static constexpr double w[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                    1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    static constexpr int opp[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
};
template <> struct Lat<3, 15> {
    static constexpr int cx[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
    static constexpr int cy[15] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1};
    static constexpr int cz[15] = {0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1};
    static constexpr double w[15] = {2.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                     1.0 / 9.0, 1.0 / 9.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                                     1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};
    static constexpr int opp[15] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13};
};
template <> struct Lat<3, 19> {
    static constexpr int cx[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
    static constexpr int cy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
    static constexpr int cz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
    static constexpr double w[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                                     1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                     1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                     1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    static constexpr int opp[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
};
template <> struct Lat<3, 27> {
    static constexpr int cx[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1,
                                   -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
    static constexpr int cy[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1,
                                   1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
    static constexpr int cz[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0,
                                   0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
    static constexpr double w[27] = {
        8.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,
        1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,
        1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 216.0, 1.0 / 216.0,
        1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0};
    static constexpr int opp[27] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14,
                                    13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25};
};

constexpr double kCs2inv = 3.0;  // LatticeDescriptor.H:29 (cs2inv)

struct State {
    orc_desc d;
    int gx, gy, gz, gk;
    long long gcells;
    int periodic[3];
    int rtype[27];
    double rrho[27];
    double rU[27][3];
    std::vector<double> fin, fout;
    // Interior obstacles (no counterpart in the reference): solid[cell] = 1,
    // valid cells x fastest; empty when the domain has none.
    std::vector<unsigned char> solid;

    long long at(int i, int j, int k) const {
        return ((long long)(k + gk) * gy + (j + 1)) * gx + (i + 1);
    }
    bool inDomain(int i, int j, int k) const {
        return i >= 0 && i < d.n[0] && j >= 0 && j < d.n[1] && k >= 0 && k < d.n[2];
    }
    // Is the upstream cell (i, j, k) (possibly a periodic image) an obstacle?
    // Cells beyond a non-periodic face belong to the face's boundary rule.
    bool solidAt(int i, int j, int k) const {
        if (solid.empty()) return false;
        int g[3] = {i, j, k};
        for (int dd = 0; dd < 3; ++dd) {
            if (g[dd] >= 0 && g[dd] < d.n[dd]) continue;
            if (!periodic[dd]) return false;
            g[dd] = g[dd] < 0 ? g[dd] + d.n[dd] : g[dd] - d.n[dd];
        }
        return solid[((long long)g[2] * d.n[1] + g[1]) * d.n[0] + g[0]] != 0;
    }
};

// Pull of cell (i, j, k) (streamCell, Streaming.H:20-35) with the interior
// obstacle rule: a population whose upstream cell is solid takes the cell's
// own opposite population, the BounceBack rule of BounceBack.H:36-63 with
// U = 0 applied at an obstacle face.
template <int D, int Q, class Lt>
inline void pullCell(const State& s, const double* fin, int i, int j, int k, const long long* off, double* f) {
    const long long c = s.at(i, j, k);
    for (int n = 0; n < Q; ++n) {
        if (s.solidAt(i - Lt::cx[n], j - Lt::cy[n], k - (D == 3 ? Lt::cz[n] : 0)))
            f[n] = fin[(long long)Lt::opp[n] * s.gcells + c];
        else
            f[n] = fin[c + off[n]];
    }
}

// ---------------------------------------------------------------------------
// Per-cell arithmetic: Macroscopic.H:36-45,158-204,241-278, Equilibrium.H:28-57,
// Collision.H:21-76.  Expression shapes are kept identical to the reference so
// the operation order (and hence rounding) is the same.
// ---------------------------------------------------------------------------
template <int D, int Q>
inline void velocity(const double* f, double rho, const double* F, bool forced, double* u) {
    using L = Lat<D, Q>;
    double ux = 0., uy = 0., uz = 0.;
    for (int n = 0; n < Q; ++n) {
        ux += L::cx[n] * f[n];
        uy += L::cy[n] * f[n];
        if (D == 3) uz += L::cz[n] * f[n];
    }
    if (!forced) {
        u[0] = ux / rho; u[1] = uy / rho;
        if (D == 3) u[2] = uz / rho;
    } else {
        u[0] = (ux + 0.5 * F[0]) / rho;
        u[1] = (uy + 0.5 * F[1]) / rho;
        if (D == 3) u[2] = (uz + 0.5 * F[2]) / rho;
    }
}

template <int D, int Q>
inline double feq(double rho, const double* u, int n) {
    using L = Lat<D, Q>;
    double u_sq, cdotu;
    if (D == 2) {
        u_sq = u[0] * u[0] + u[1] * u[1];
        cdotu = L::cx[n] * u[0] + L::cy[n] * u[1];
    } else {
        u_sq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        cdotu = L::cx[n] * u[0] + L::cy[n] * u[1] + L::cz[n] * u[2];
    }
    return L::w[n] * rho *
           (1 + kCs2inv * cdotu + 0.5 * kCs2inv * kCs2inv * cdotu * cdotu - 0.5 * kCs2inv * u_sq);
}

template <int D, int Q>
inline double guo(int n, const double* u, const double* F, double omega) {
    using L = Lat<D, Q>;
    double cdotF, cdotu, udotF;
    if (D == 2) {
        cdotF = L::cx[n] * F[0] + L::cy[n] * F[1];
        cdotu = L::cx[n] * u[0] + L::cy[n] * u[1];
        udotF = u[0] * F[0] + u[1] * F[1];
    } else {
        cdotF = L::cx[n] * F[0] + L::cy[n] * F[1] + L::cz[n] * F[2];
        cdotu = L::cx[n] * u[0] + L::cy[n] * u[1] + L::cz[n] * u[2];
        udotF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
    }
    return (1.0 - 0.5 * omega) * L::w[n] * kCs2inv * (cdotF + kCs2inv * cdotu * cdotF - udotF);
}

inline double bgk(double f, double fe, double omega) { return (1 - omega) * f + omega * fe; }

// pullCollideFusedArr, Collision.cpp:18-92 (unforced and forced variants).
template <int D, int Q, bool FORCED>
void pullCollide(State& s, int nthreads) {
    using L = Lat<D, Q>;
    const double omega = s.d.omega;
    const double* F = s.d.F;
    const double* fin = s.fin.data();
    double* fout = s.fout.data();
    const long long G = s.gcells;
    const int nx = s.d.n[0], ny = s.d.n[1], nz = s.d.n[2];
    long long off[Q];
    for (int n = 0; n < Q; ++n)
        off[n] = (long long)n * G - ((long long)L::cz[n] * s.gy + L::cy[n]) * s.gx - L::cx[n];
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads)
    for (int k = 0; k < nz; ++k) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const long long c = s.at(i, j, k);
                double f[Q];
                if (!s.solid.empty()) {
                    if (s.solid[((long long)k * ny + j) * nx + i]) {  // obstacle: rest state
                        for (int n = 0; n < Q; ++n) fout[(long long)n * G + c] = L::w[n];
                        continue;
                    }
                    pullCell<D, Q, L>(s, fin, i, j, k, off, f);
                } else {
                    for (int n = 0; n < Q; ++n) f[n] = fin[c + off[n]];  // streamCell, Streaming.H:20-35
                }
                double rho = 0.;
                for (int n = 0; n < Q; ++n) rho += f[n];
                double u[3];
                velocity<D, Q>(f, rho, F, FORCED, u);
                for (int n = 0; n < Q; ++n) {
                    const double fe = feq<D, Q>(rho, u, n);
                    double o = bgk(f[n], fe, omega);
                    if (FORCED) o = o + guo<D, Q>(n, u, F, omega);
                    fout[(long long)n * G + c] = o;
                }
            }
        }
    }
}

// MultiFab::FillBoundary(periodicity) for a single box: every ghost cell whose
// periodic image is a valid cell receives all Q components of that image
// (SimulationSetup.cpp:227).
template <int D, int Q>
void fillPeriodic(State& s) {
    const int kl = (D == 3) ? -1 : 0, kh = (D == 3) ? s.d.n[2] : 0;
    const long long G = s.gcells;
    double* f = s.fin.data();
    for (int k = kl; k <= kh; ++k)
        for (int j = -1; j <= s.d.n[1]; ++j)
            for (int i = -1; i <= s.d.n[0]; ++i) {
                if (s.inDomain(i, j, k)) continue;
                int g[3] = {i, j, k};
                bool ok = true;
                for (int dd = 0; dd < D; ++dd) {
                    if (g[dd] < 0 || g[dd] >= s.d.n[dd]) {
                        if (!s.periodic[dd]) { ok = false; break; }
                        g[dd] = (g[dd] < 0) ? g[dd] + s.d.n[dd] : g[dd] - s.d.n[dd];
                    }
                }
                if (!ok) continue;
                const long long dst = s.at(i, j, k), src = s.at(g[0], g[1], g[2]);
                for (int n = 0; n < Q; ++n) f[n * G + dst] = f[n * G + src];
            }
}

// BCManager<L>::operator(), BoundaryConditions.H:124-189, dispatching to the
// ghost-fill kernels of BCTypes/*.H.
template <int D, int Q>
void applyBC(State& s, int i, int j, int k) {
    using L = Lat<D, Q>;
    const long long G = s.gcells;
    double* f = s.fin.data();
    int iv[3] = {i, j, k};
    int code[3] = {0, 0, 0};
    for (int dd = 0; dd < D; ++dd) {
        if (iv[dd] < 0) code[dd] = -1;
        else if (iv[dd] > s.d.n[dd] - 1) code[dd] = 1;
        else code[dd] = 0;
        if (s.periodic[dd]) code[dd] = 0;
    }
    bool all_zero = true;
    for (int dd = 0; dd < D; ++dd) if (code[dd] != 0) all_zero = false;
    if (all_zero) return;
    int idx = 0, p3 = 1;
    for (int dd = 0; dd < D; ++dd) { idx += (code[dd] + 1) * p3; p3 *= 3; }
    const int type = s.rtype[idx];
    if (type == BC_PERIODIC) return;
    const long long g = s.at(i, j, k);

    if (type == BC_MOVING || type == BC_NOSLIP || type == BC_INFLOW) {
        // BounceBack<L>::apply, BCTypes/BounceBack.H:36-63.  NoSlip passes
        // rho = 1 and U = 0 (NoSlipKernel.H:20-28).
        double rho = 1;
        double U[3] = {0., 0., 0.};
        if (type != BC_NOSLIP) {
            rho = s.rrho[idx];
            U[0] = s.rU[idx][0]; U[1] = s.rU[idx][1]; U[2] = s.rU[idx][2];
        }
        for (int n = 0; n < Q; ++n) {
            const int si = i + L::cx[n], sj = j + L::cy[n], sk = k + (D == 3 ? L::cz[n] : 0);
            if (!s.inDomain(si, sj, sk)) continue;
            const int o = L::opp[n];
            double cdotu;
            if (D == 2) cdotu = L::cx[o] * U[0] + L::cy[o] * U[1];
            else cdotu = L::cx[o] * U[0] + L::cy[o] * U[1] + L::cz[o] * U[2];
            const double contrib = -2. * rho * L::w[o] * cdotu * kCs2inv;
            f[n * G + g] = f[o * G + s.at(si, sj, sk)] + contrib;
        }
    } else if (type == BC_OUTFLOW) {
        // OutflowKernel<L>::apply, BCTypes/OutflowKernel.H:26-38.
        for (int n = 0; n < Q; ++n) {
            const int si = i + L::cx[n], sj = j + L::cy[n], sk = k + (D == 3 ? L::cz[n] : 0);
            if (!s.inDomain(si, sj, sk)) continue;
            f[n * G + g] = f[n * G + s.at(si, sj, sk)];
        }
    } else if (type == BC_PRESSURE) {
        // PressureOutletKernel<L>::apply, BCTypes/PressureOutletKernel.H:29-64.
        const double rho_out = s.rrho[idx];
        for (int n = 0; n < Q; ++n) {
            const int si = i + L::cx[n], sj = j + L::cy[n], sk = k + (D == 3 ? L::cz[n] : 0);
            if (!s.inDomain(si, sj, sk)) continue;
            const long long src = s.at(si, sj, sk);
            double rho = 0.0;
            double jv[3] = {0., 0., 0.};
            for (int m = 0; m < Q; ++m) {
                const double fm = f[m * G + src];
                rho += fm;
                jv[0] += L::cx[m] * fm;
                jv[1] += L::cy[m] * fm;
                if (D == 3) jv[2] += L::cz[m] * fm;
            }
            const double inv_rho = 1.0 / rho;
            double cu, uu;
            if (D == 2) {
                cu = (L::cx[n] * jv[0] + L::cy[n] * jv[1]) * inv_rho;
                uu = (jv[0] * jv[0] + jv[1] * jv[1]) * inv_rho * inv_rho;
            } else {
                cu = (L::cx[n] * jv[0] + L::cy[n] * jv[1] + L::cz[n] * jv[2]) * inv_rho;
                uu = (jv[0] * jv[0] + jv[1] * jv[1] + jv[2] * jv[2]) * inv_rho * inv_rho;
            }
            const double feq_even =
                L::w[n] * rho_out * (1.0 + 0.5 * cu * cu * kCs2inv * kCs2inv - 0.5 * uu * kCs2inv);
            f[n * G + g] = -f[L::opp[n] * G + src] + 2.0 * feq_even;
        }
    }
}

// SimulationImpl::fillGhostCells, SimulationSetup.cpp:222-234.
template <int D, int Q>
void fillGhosts(State& s) {
    fillPeriodic<D, Q>(s);
    const int kl = (D == 3) ? -1 : 0, kh = (D == 3) ? s.d.n[2] : 0;
    for (int k = kl; k <= kh; ++k)
        for (int j = -1; j <= s.d.n[1]; ++j)
            for (int i = -1; i <= s.d.n[0]; ++i) {
                if (s.inDomain(i, j, k)) continue;
                applyBC<D, Q>(s, i, j, k);
            }
}

// setInitialConditions, SimulationSetup.cpp:201-219 with initVelCorrection
// (Macroscopic.cpp:164-181), computeEquilibriumMF (Equilibrium.cpp:46-67) and
// computeMacroscopic (Macroscopic.cpp:139-162).
template <int D, int Q>
void initFields(State& s, double* rho, double* u) {
    const long long N = (long long)s.d.n[0] * s.d.n[1] * s.d.n[2];
    const long long G = s.gcells;
    double* f = s.fin.data();
    if (s.d.forced)
        for (long long c = 0; c < N; ++c)
            for (int dd = 0; dd < D; ++dd) u[dd * N + c] -= 0.5 * s.d.F[dd] / rho[c];
    long long c = 0;
    for (int k = 0; k < s.d.n[2]; ++k)
        for (int j = 0; j < s.d.n[1]; ++j)
            for (int i = 0; i < s.d.n[0]; ++i, ++c) {
                double uc[3] = {u[c], u[N + c], D == 3 ? u[2 * N + c] : 0.0};
                const long long g = s.at(i, j, k);
                for (int n = 0; n < Q; ++n) f[n * G + g] = feq<D, Q>(rho[c], uc, n);
            }
    if (s.d.forced) {
        c = 0;
        for (int k = 0; k < s.d.n[2]; ++k)
            for (int j = 0; j < s.d.n[1]; ++j)
                for (int i = 0; i < s.d.n[0]; ++i, ++c) {
                    const long long g = s.at(i, j, k);
                    double fl[Q];
                    for (int n = 0; n < Q; ++n) fl[n] = f[n * G + g];
                    double r = 0.;
                    for (int n = 0; n < Q; ++n) r += fl[n];
                    double uc[3];
                    velocity<D, Q>(fl, r, s.d.F, true, uc);
                    rho[c] = r;
                    for (int dd = 0; dd < D; ++dd) u[dd * N + c] = uc[dd];
                }
    }
    fillGhosts<D, Q>(s);
}

// updateMacroscopic, SimulationSetup.cpp:142-166: streamMF (Streaming.cpp:15-49)
// into scratch, then computeMacroscopic (Macroscopic.cpp:115-162).
template <int D, int Q>
void moments(State& s, double* rho, double* u) {
    using L = Lat<D, Q>;
    const long long N = (long long)s.d.n[0] * s.d.n[1] * s.d.n[2];
    const long long G = s.gcells;
    const double* fin = s.fin.data();
    long long off[Q];
    for (int n = 0; n < Q; ++n)
        off[n] = (long long)n * G - ((long long)(D == 3 ? L::cz[n] : 0) * s.gy + L::cy[n]) * s.gx - L::cx[n];
    long long c = 0;
    for (int k = 0; k < s.d.n[2]; ++k)
        for (int j = 0; j < s.d.n[1]; ++j)
            for (int i = 0; i < s.d.n[0]; ++i, ++c) {
                double f[Q];
                pullCell<D, Q, L>(s, fin, i, j, k, off, f);
                double r = 0.;
                for (int n = 0; n < Q; ++n) r += f[n];
                double uc[3];
                velocity<D, Q>(f, r, s.d.F, s.d.forced != 0, uc);
                rho[c] = r;
                for (int dd = 0; dd < D; ++dd) u[dd * N + c] = uc[dd];
            }
}

template <int D, int Q>
int dispatchStep(State& s, int nsteps, int nthreads) {
    for (int t = 0; t < nsteps; ++t) {
        if (s.d.forced) pullCollide<D, Q, true>(s, nthreads);
        else pullCollide<D, Q, false>(s, nthreads);
        std::swap(s.fin, s.fout);  // SimulationSetup.cpp:132
        fillGhosts<D, Q>(s);
    }
    return 0;
}

#define ORC_DISPATCH(s, call)                                             \
    do {                                                                  \
        if ((s).d.dim == 2 && (s).d.q == 9) { call(2, 9); }               \
        else if ((s).d.dim == 3 && (s).d.q == 15) { call(3, 15); }        \
        else if ((s).d.dim == 3 && (s).d.q == 19) { call(3, 19); }        \
        else if ((s).d.dim == 3 && (s).d.q == 27) { call(3, 27); }        \
        else return -1;                                                   \
    } while (0)

// hasConflictingBC, BoundaryConditions.cpp:37-57.
bool conflicting(const int* types, int nt) {
    bool in = false, out = false, pr = false;
    int moving = 0;
    for (int a = 0; a < nt; ++a) {
        if (types[a] == BC_INFLOW) in = true;
        if (types[a] == BC_OUTFLOW) out = true;
        if (types[a] == BC_PRESSURE) pr = true;
        if (types[a] == BC_MOVING) moving++;
    }
    return ((int)in + (int)out + (int)pr) > 1 || moving > 1;
}

// bcRank, BoundaryConditions.H:82-92.
int rankOf(int t) {
    switch (t) {
        case BC_NOSLIP: return 3;
        case BC_MOVING: return 2;
        case BC_INFLOW: return 1;
        case BC_OUTFLOW: return 0;
        case BC_PRESSURE: return 0;
        default: return -1;
    }
}

// BCManager::finalize + resolveBC, BoundaryConditions.cpp:59-155.
int resolveTable(const orc_desc* d, int* type, double* rho, double* U) {
    const int D = d->dim;
    int total = 1;
    for (int dd = 0; dd < D; ++dd) total *= 3;
    for (int idx = 0; idx < 27; ++idx) {
        type[idx] = BC_PERIODIC; rho[idx] = 1.0;
        U[3 * idx] = U[3 * idx + 1] = U[3 * idx + 2] = 0.0;
    }
    for (int idx = 0; idx < total; ++idx) {
        int code[3] = {0, 0, 0}, tmp = idx;
        for (int dd = 0; dd < D; ++dd) { code[dd] = (tmp % 3) - 1; tmp /= 3; }
        bool all_zero = true;
        for (int dd = 0; dd < D; ++dd) if (code[dd] != 0) all_zero = false;
        if (all_zero) continue;
        int ft[3]; double fr[3]; double fu[3][3]; int nf = 0;
        for (int dd = 0; dd < D; ++dd) {
            if (code[dd] == 0) continue;
            const int fi = 2 * dd + (code[dd] < 0 ? 0 : 1);
            // A face is Periodic when its own name is Periodic (BCManager keeps
            // m_face_bc = Periodic for it, SimulationSetup.cpp:256-262).
            if (d->face_type[fi] == BC_PERIODIC) continue;
            ft[nf] = d->face_type[fi];
            fr[nf] = d->face_rho[fi];
            for (int c = 0; c < 3; ++c) fu[nf][c] = d->face_U[fi][c];
            ++nf;
        }
        if (nf == 0) continue;
        if (conflicting(ft, nf)) return 1;
        int max_rank = -1;
        for (int a = 0; a < nf; ++a) max_rank = std::max(max_rank, rankOf(ft[a]));
        int winner = 0;
        for (int a = 0; a < nf; ++a) if (rankOf(ft[a]) == max_rank) { winner = ft[a]; break; }
        double sum_rho = 0;
        double sum_U[3] = {0., 0., 0.};
        int count = 0;
        for (int a = 0; a < nf; ++a) {
            if (ft[a] == winner) {
                sum_rho += fr[a];
                for (int c = 0; c < D; ++c) sum_U[c] += fu[a][c];
                ++count;
            }
        }
        type[idx] = winner;
        if (count > 0) {
            rho[idx] = sum_rho / count;
            for (int c = 0; c < D; ++c) U[3 * idx + c] = sum_U[c] / count;
        }
    }
    return 0;
}

}  // namespace

extern "C" {

int orc_units(const orc_units_in* in, orc_units_out* out, int nacc, const double* accel_phys,
              double* accel_lat, int nvel, const double* vel_phys, double* vel_lat, int nrho,
              const double* rho_phys, double* rho_lat) {
    // UnitConverter::setGridResolution, Units.cpp:131-167.
    const int D = in->dim;
    int max_N = in->ncells[0];
    for (int dd = 0; dd < D; ++dd) max_N = (in->ncells[dd] > max_N) ? in->ncells[dd] : max_N;
    double domLength[3] = {0., 0., 0.}, gridRes[3] = {0., 0., 0.};
    double max_L = -1;
    for (int dd = 0; dd < D; ++dd) {
        domLength[dd] = in->prob_hi[dd] - in->prob_lo[dd];
        max_L = (domLength[dd] > max_L) ? domLength[dd] : max_L;
        gridRes[dd] = domLength[dd] / double(in->ncells[dd]);
    }
    const double tol = 1.0e-12;
    if (!(std::abs(gridRes[0] - gridRes[1]) < tol)) return 2;
    if (D == 3) {
        if (!(std::abs(gridRes[0] - gridRes[2]) < tol)) return 2;
        if (!(std::abs(gridRes[1] - gridRes[2]) < tol)) return 2;
    }
    const double dx = max_L / double(max_N);
    // UnitConverter ctor, Units.cpp:20-109.
    double Re, nu;
    if (in->has_nu) {
        nu = in->nu_phys;
        Re = in->ref_velocity * in->ref_length / nu;
        if (in->has_Re) return 3;
    } else if (in->has_Re) {
        Re = in->Re;
        nu = in->ref_velocity * in->ref_length / Re;
    } else {
        return 3;
    }
    const double cs2 = 1.0 / 3.0;
    double u_lat;
    if (in->has_tau) {
        const double nu_lat_from_tau = (in->tau - 0.5) * cs2;
        const double u_lat_from_tau = nu_lat_from_tau * in->ref_velocity * dx / nu;
        if (in->has_u_lat) return 4;
        u_lat = u_lat_from_tau;
    } else if (in->has_u_lat) {
        u_lat = in->u_lat;
    } else {
        u_lat = 0.1;
    }
    const double dt = u_lat * dx / in->ref_velocity;
    const double nu_lat = nu * dt / (dx * dx);
    const double tau = 0.5 + nu_lat / cs2;
    out->dx = dx; out->dt = dt; out->u_lat = u_lat; out->nu_lat = nu_lat;
    out->tau = tau; out->Re = Re; out->nu_phys = nu;
    out->omega = 1.0 / tau;  // SimulationSetup.cpp:54
    // Conversions, Units.cpp:169-176.
    for (int a = 0; a < nacc; ++a) accel_lat[a] = accel_phys[a] * dt * dt / dx;
    for (int a = 0; a < nvel; ++a) vel_lat[a] = vel_phys[a] * dt / dx;
    for (int a = 0; a < nrho; ++a) rho_lat[a] = rho_phys[a] / in->ref_density;
    if (!((tau > 0.5) && (tau < 2.0))) return 5;
    if (!(u_lat < 0.3)) return 6;
    return 0;
}

int orc_resolve_bc(const orc_desc* d, int* type, double* rho, double* U) {
    return resolveTable(d, type, rho, U);
}

void* orc_create(const orc_desc* d) {
    if (!d) return nullptr;
    if (!((d->dim == 2 && d->q == 9) || (d->dim == 3 && (d->q == 15 || d->q == 19 || d->q == 27))))
        return nullptr;
    for (int dd = 0; dd < 3; ++dd) if (d->n[dd] < 1) return nullptr;
    if (d->dim == 2 && d->n[2] != 1) return nullptr;
    State* s = new State();
    s->d = *d;
    s->gx = d->n[0] + 2;
    s->gy = d->n[1] + 2;
    s->gz = (d->dim == 3) ? d->n[2] + 2 : 1;
    s->gk = (d->dim == 3) ? 1 : 0;
    s->gcells = (long long)s->gx * s->gy * s->gz;
    for (int dd = 0; dd < 3; ++dd)
        s->periodic[dd] = (dd < d->dim) && d->face_type[2 * dd] == BC_PERIODIC;  // GeometryHandler.cpp:39-48
    // A "Periodic" name on a face whose direction is not periodic aborts in
    // buildBCManager (SimulationSetup.cpp:256-260).
    for (int dd = 0; dd < d->dim; ++dd)
        if (d->face_type[2 * dd + 1] == BC_PERIODIC && !s->periodic[dd]) { delete s; return nullptr; }
    if (resolveTable(d, s->rtype, s->rrho, &s->rU[0][0]) != 0) { delete s; return nullptr; }
    const double nan = std::nan("");
    s->fin.assign((size_t)d->q * s->gcells, nan);
    s->fout.assign((size_t)d->q * s->gcells, nan);
    return s;
}

void orc_destroy(void* p) { delete static_cast<State*>(p); }
long long orc_ncells(void* p) { auto* s = static_cast<State*>(p); return (long long)s->d.n[0] * s->d.n[1] * s->d.n[2]; }
long long orc_nghost_cells(void* p) { return static_cast<State*>(p)->gcells; }

int orc_set_f(void* p, const double* f) {
    auto* s = static_cast<State*>(p);
    long long c = 0;
    for (int n = 0; n < s->d.q; ++n)
        for (int k = 0; k < s->d.n[2]; ++k)
            for (int j = 0; j < s->d.n[1]; ++j)
                for (int i = 0; i < s->d.n[0]; ++i, ++c) s->fin[n * s->gcells + s->at(i, j, k)] = f[c];
    return 0;
}

int orc_get_f(void* p, double* f) {
    auto* s = static_cast<State*>(p);
    long long c = 0;
    for (int n = 0; n < s->d.q; ++n)
        for (int k = 0; k < s->d.n[2]; ++k)
            for (int j = 0; j < s->d.n[1]; ++j)
                for (int i = 0; i < s->d.n[0]; ++i, ++c) f[c] = s->fin[n * s->gcells + s->at(i, j, k)];
    return 0;
}

int orc_set_f_ghost(void* p, const double* f) {
    auto* s = static_cast<State*>(p);
    std::memcpy(s->fin.data(), f, sizeof(double) * s->fin.size());
    return 0;
}

int orc_get_f_ghost(void* p, double* f) {
    auto* s = static_cast<State*>(p);
    std::memcpy(f, s->fin.data(), sizeof(double) * s->fin.size());
    return 0;
}

int orc_fill_ghosts(void* p) {
    auto& s = *static_cast<State*>(p);
#define ORC_CALL(D, Q) fillGhosts<D, Q>(s)
    ORC_DISPATCH(s, ORC_CALL);
#undef ORC_CALL
    return 0;
}

int orc_step(void* p, int nsteps, int nthreads) {
    auto& s = *static_cast<State*>(p);
    if (nthreads < 1) nthreads = 1;
#define ORC_CALL(D, Q) return dispatchStep<D, Q>(s, nsteps, nthreads)
    ORC_DISPATCH(s, ORC_CALL);
#undef ORC_CALL
    return 0;
}

int orc_init_fields(void* p, double* rho, double* u) {
    auto& s = *static_cast<State*>(p);
#define ORC_CALL(D, Q) initFields<D, Q>(s, rho, u)
    ORC_DISPATCH(s, ORC_CALL);
#undef ORC_CALL
    return 0;
}

int orc_set_obstacles(void* p, const unsigned char* mask) {
    auto& s = *static_cast<State*>(p);
    const long long N = (long long)s.d.n[0] * s.d.n[1] * s.d.n[2];
    if (!mask) { s.solid.clear(); return 0; }
    s.solid.assign(mask, mask + N);
    for (auto& v : s.solid) v = v ? 1 : 0;
    return 0;
}

int orc_moments(void* p, double* rho, double* u) {
    auto& s = *static_cast<State*>(p);
#define ORC_CALL(D, Q) moments<D, Q>(s, rho, u)
    ORC_DISPATCH(s, ORC_CALL);
#undef ORC_CALL
    return 0;
}

}  // extern "C"
