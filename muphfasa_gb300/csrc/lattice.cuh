// lattice.cuh -- compile-time velocity sets, usable from host and device.
//
// The q ordering, velocities, weights and opposite tables are those of the
// reference's LatticeDescriptor.H:23-263 (D2Q9, D3Q15, D3Q19, D3Q27): the
// population index is part of the data layout shared with the reference, so
// it has to be the same.  Weights are the same rational constants rounded to
// double.
#pragma once

#define MPH_HD __host__ __device__ __forceinline__

namespace mph {

template <int Q> struct Lat;

template <> struct Lat<9> {
    static constexpr int D = 2, Q = 9;
    // exact inverse of the weight (w is 4/9, 1/9, 1/36, ...; 1/w is representable)
    static MPH_HD constexpr double iw(int n) { return n == 0 ? 2.25 : (n < 5 ? 9.0 : 36.0); }
    static MPH_HD constexpr int cx(int n) { constexpr int t[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1}; return t[n]; }
    static MPH_HD constexpr int cy(int n) { constexpr int t[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1}; return t[n]; }
    static MPH_HD constexpr int cz(int) { return 0; }
    static MPH_HD constexpr int opp(int n) { constexpr int t[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6}; return t[n]; }
    static MPH_HD constexpr double w(int n) {
        constexpr double t[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
        return t[n];
    }
};

template <> struct Lat<15> {
    static constexpr int D = 3, Q = 15;
    // exact inverse of the weight (w is 4/9, 1/9, 1/36, ...; 1/w is representable)
    static MPH_HD constexpr double iw(int n) { return n == 0 ? 4.5 : (n < 7 ? 9.0 : 72.0); }
    static MPH_HD constexpr int cx(int n) { constexpr int t[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1}; return t[n]; }
    static MPH_HD constexpr int cy(int n) { constexpr int t[15] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1}; return t[n]; }
    static MPH_HD constexpr int cz(int n) { constexpr int t[15] = {0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1}; return t[n]; }
    static MPH_HD constexpr int opp(int n) { constexpr int t[15] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13}; return t[n]; }
    static MPH_HD constexpr double w(int n) {
        constexpr double t[15] = {2.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                                  1.0 / 9.0, 1.0 / 9.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                                  1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};
        return t[n];
    }
};

template <> struct Lat<19> {
    static constexpr int D = 3, Q = 19;
    // exact inverse of the weight (w is 4/9, 1/9, 1/36, ...; 1/w is representable)
    static MPH_HD constexpr double iw(int n) { return n == 0 ? 3.0 : (n < 7 ? 18.0 : 36.0); }
    static MPH_HD constexpr int cx(int n) { constexpr int t[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0}; return t[n]; }
    static MPH_HD constexpr int cy(int n) { constexpr int t[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1}; return t[n]; }
    static MPH_HD constexpr int cz(int n) { constexpr int t[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1}; return t[n]; }
    static MPH_HD constexpr int opp(int n) { constexpr int t[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17}; return t[n]; }
    static MPH_HD constexpr double w(int n) {
        constexpr double t[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                                  1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                  1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                                  1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
        return t[n];
    }
};

template <> struct Lat<27> {
    static constexpr int D = 3, Q = 27;
    // exact inverse of the weight (w is 4/9, 1/9, 1/36, ...; 1/w is representable)
    static MPH_HD constexpr double iw(int n) { return n == 0 ? 3.375 : (n < 7 ? 13.5 : (n < 19 ? 54.0 : 216.0)); }
    static MPH_HD constexpr int cx(int n) {
        constexpr int t[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
        return t[n];
    }
    static MPH_HD constexpr int cy(int n) {
        constexpr int t[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
        return t[n];
    }
    static MPH_HD constexpr int cz(int n) {
        constexpr int t[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
        return t[n];
    }
    static MPH_HD constexpr int opp(int n) {
        constexpr int t[27] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25};
        return t[n];
    }
    static MPH_HD constexpr double w(int n) {
        constexpr double t[27] = {8.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,  2.0 / 27.0,
                                  2.0 / 27.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,
                                  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,  1.0 / 54.0,
                                  1.0 / 54.0,  1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0,
                                  1.0 / 216.0, 1.0 / 216.0, 1.0 / 216.0};
        return t[n];
    }
};

// Weight class of population n: |c_n|^2 (0 rest, 1 face, 2 edge, 3 corner).
template <int Q>
MPH_HD constexpr int wclass(int n) {
    return Lat<Q>::cx(n) * Lat<Q>::cx(n) + Lat<Q>::cy(n) * Lat<Q>::cy(n) + Lat<Q>::cz(n) * Lat<Q>::cz(n);
}

}  // namespace mph
