// mph_amrex_standin.H -- a small, project-written stand-in for the part of the
// AMReX container API that the reference's LBM sources (src/LBM/*.H, *.cpp)
// touch, so that those sources compile unchanged on a host that has no AMReX.
// Single box, CPU loops, no MPI, no GPU.  Used only to build the reference
// checker under oracle/_ref/ (oracle/build_ref.sh); never part of the product.
//
// AMREX_SPACEDIM must be defined (2 or 3) by the compiler command line.
#ifndef MPH_AMREX_STANDIN_H
#define MPH_AMREX_STANDIN_H

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#ifndef AMREX_SPACEDIM
#error "AMREX_SPACEDIM must be defined"
#endif
#ifdef _OPENMP
#include <omp.h>
#endif

#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_DEVICE
// As AMReX defines it for GCC/Clang: the reference's per-cell helpers
// (lattice accessors, streamCell, equilibrium, Guo term) must inline into the
// cell loop so their constant tables fold.
#define AMREX_FORCE_INLINE inline __attribute__((always_inline))
#if (AMREX_SPACEDIM == 2)
#define AMREX_D_DECL(a, b, c) a, b
#define AMREX_D_TERM(a, b, c) a b
#else
#define AMREX_D_DECL(a, b, c) a, b, c
#define AMREX_D_TERM(a, b, c) a b c
#endif
#define BL_PROFILE(name)
#define AMREX_ALWAYS_ASSERT_WITH_MESSAGE(cond, msg) \
    do { if (!(cond)) { ::amrex::Abort(msg); } } while (0)

namespace amrex {

using Real = double;
using Long = long long;

// Errors surface as exceptions so the checker's C entry points can turn a
// reference abort into a status code.
[[noreturn]] inline void Abort(const std::string& msg) { throw std::runtime_error(msg); }
[[noreturn]] inline void Abort(const char* msg) { throw std::runtime_error(msg ? msg : "abort"); }

template <class... Ts> inline void ignore_unused(const Ts&...) {}

template <class T> using Vector = std::vector<T>;
template <class T, std::size_t N> using Array = std::array<T, N>;

template <class T, int N>
struct GpuArray {
    T arr[N];
    T& operator[](int i) noexcept { return arr[i]; }
    const T& operator[](int i) const noexcept { return arr[i]; }
    void fill(const T& v) noexcept { for (int i = 0; i < N; ++i) arr[i] = v; }
};

struct IntVect {
    int v[3] = {0, 0, 0};
    IntVect() = default;
    explicit IntVect(int a) { for (int d = 0; d < AMREX_SPACEDIM; ++d) v[d] = a; }
#if (AMREX_SPACEDIM == 2)
    IntVect(int a, int b) { v[0] = a; v[1] = b; v[2] = 0; }
#else
    IntVect(int a, int b, int c) { v[0] = a; v[1] = b; v[2] = c; }
#endif
    int& operator[](int d) noexcept { return v[d]; }
    int operator[](int d) const noexcept { return v[d]; }
    IntVect operator+(const IntVect& o) const { IntVect r; for (int d = 0; d < 3; ++d) r.v[d] = v[d] + o.v[d]; return r; }
    IntVect operator-(const IntVect& o) const { IntVect r; for (int d = 0; d < 3; ++d) r.v[d] = v[d] - o.v[d]; return r; }
};

class Box {
public:
    Box() = default;
    Box(const IntVect& lo, const IntVect& hi) : m_lo(lo), m_hi(hi) {}
    const IntVect& smallEnd() const noexcept { return m_lo; }
    const IntVect& bigEnd() const noexcept { return m_hi; }
    int smallEnd(int d) const noexcept { return m_lo[d]; }
    int bigEnd(int d) const noexcept { return m_hi[d]; }
    int length(int d) const noexcept { return m_hi[d] - m_lo[d] + 1; }
    bool contains(const IntVect& p) const noexcept {
        for (int d = 0; d < AMREX_SPACEDIM; ++d) if (p[d] < m_lo[d] || p[d] > m_hi[d]) return false;
        return true;
    }
    bool contains(const Box& b) const noexcept { return contains(b.m_lo) && contains(b.m_hi); }
private:
    IntVect m_lo, m_hi;
};

inline Box grow(const Box& b, int n) {
    IntVect lo = b.smallEnd(), hi = b.bigEnd();
    for (int d = 0; d < AMREX_SPACEDIM; ++d) { lo[d] -= n; hi[d] += n; }
    return Box(lo, hi);
}

// Array4: i fastest, then j, k, component n.  begin/end follow AMReX
// (end exclusive); 2-D boxes have a single k plane.
template <class T>
struct Array4 {
    T* p = nullptr;
    Long jstride = 0, kstride = 0, nstride = 0;
    int begin[3] = {0, 0, 0};
    int end[3] = {1, 1, 1};
    int ncomp = 1;

    Array4() = default;
    Array4(T* ptr, const Box& b, int nc) : p(ptr), ncomp(nc) {
        for (int d = 0; d < AMREX_SPACEDIM; ++d) { begin[d] = b.smallEnd(d); end[d] = b.bigEnd(d) + 1; }
        jstride = end[0] - begin[0];
        kstride = jstride * (end[1] - begin[1]);
        nstride = kstride * (end[2] - begin[2]);
    }
    template <class U, class = typename std::enable_if<std::is_same<const U, T>::value>::type>
    Array4(const Array4<U>& o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), ncomp(o.ncomp) {
        for (int d = 0; d < 3; ++d) { begin[d] = o.begin[d]; end[d] = o.end[d]; }
    }
    T& operator()(int i, int j, int k) const noexcept {
        return p[(i - begin[0]) + (j - begin[1]) * jstride + (k - begin[2]) * kstride];
    }
    T& operator()(int i, int j, int k, int n) const noexcept {
        return p[(i - begin[0]) + (j - begin[1]) * jstride + (k - begin[2]) * kstride + n * nstride];
    }
    T& operator()(const IntVect& iv, int n) const noexcept { return (*this)(iv[0], iv[1], iv[2], n); }
    bool contains(int i, int j, int k) const noexcept {
        return i >= begin[0] && i < end[0] && j >= begin[1] && j < end[1] && k >= begin[2] && k < end[2];
    }
    bool contains(const IntVect& iv) const noexcept { return contains(iv[0], iv[1], iv[2]); }
};

class FArrayBox {
public:
    FArrayBox() = default;
    FArrayBox(const Box& b, int nc) { define(b, nc); }
    void define(const Box& b, int nc) {
        m_box = b; m_nc = nc;
        Long cells = 1;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) cells *= b.length(d);
        m_data.assign((std::size_t)(cells * nc), 0.0);
    }
    const Box& box() const noexcept { return m_box; }
    int nComp() const noexcept { return m_nc; }
    Array4<Real> array() { return Array4<Real>(m_data.data(), m_box, m_nc); }
    Array4<Real const> const_array() const { return Array4<Real const>(m_data.data(), m_box, m_nc); }
    Array4<Real const> array() const { return const_array(); }
    std::vector<Real>& data() { return m_data; }
private:
    Box m_box;
    int m_nc = 0;
    std::vector<Real> m_data;
};

class MultiFab;

// Iterator over the tiles of the one box.  With tiling the valid box is cut
// into tiles of full rows along x and 8 cells along each further direction
// (AMReX's default CPU tile shape), enumerated x-fastest; inside an OpenMP
// parallel region each thread takes its own contiguous share of the tiles,
// the first (tiles mod threads) threads one extra, so the reference's
// `#pragma omp parallel` MFIter loops run on every host thread.
class MFIter {
public:
    explicit MFIter(const MultiFab& mf, bool tiling = false);
    bool isValid() const noexcept { return m_i < m_end; }
    MFIter& operator++() noexcept { ++m_i; return *this; }
    int index() const noexcept { return 0; }
    Box tilebox() const;
    Box validbox() const;
    Box fabbox() const;
private:
    const MultiFab* m_mf;
    int m_i = 0, m_end = 1;
    int m_nt[3] = {1, 1, 1};  // tiles per direction
    int m_ts[3] = {0, 0, 0};  // tile extent per direction (0: whole box)
};

inline bool TilingIfNotGPU() { return true; }

// A single-box MultiFab: valid box plus nGhost layers (no k ghosts in 2-D).
class MultiFab {
public:
    MultiFab() = default;
    MultiFab(const Box& valid, int ncomp, int ngrow) { define(valid, ncomp, ngrow); }
    void define(const Box& valid, int ncomp, int ngrow) {
        m_valid = valid; m_ngrow = ngrow;
        m_fab.define(grow(valid, ngrow), ncomp);
    }
    FArrayBox& operator[](const MFIter&) { return m_fab; }
    const FArrayBox& operator[](const MFIter&) const { return m_fab; }
    Array4<Real> array(const MFIter&) { return m_fab.array(); }
    Array4<Real const> const_array(const MFIter&) const { return m_fab.const_array(); }
    Array4<Real const> array(const MFIter&) const { return m_fab.const_array(); }
    const Box& validBox() const noexcept { return m_valid; }
    int nComp() const noexcept { return m_fab.nComp(); }
    int nGrow() const noexcept { return m_ngrow; }
    FArrayBox& fab() { return m_fab; }
    const FArrayBox& fab() const { return m_fab; }
    void mult(Real v) { for (auto& x : m_fab.data()) x *= v; }
    void setVal(Real v) { for (auto& x : m_fab.data()) x = v; }
private:
    Box m_valid;
    int m_ngrow = 0;
    FArrayBox m_fab;
};

inline MFIter::MFIter(const MultiFab& mf, bool tiling) : m_mf(&mf) {
    const Box& v = mf.validBox();
    int total = 1;
    if (tiling) {
        for (int d = 1; d < AMREX_SPACEDIM; ++d) {
            m_ts[d] = 8;
            m_nt[d] = (v.length(d) + 7) / 8;
            total *= m_nt[d];
        }
    }
    int first = 0, count = total;
#ifdef _OPENMP
    if (omp_in_parallel()) {
        const int nth = omp_get_num_threads(), tid = omp_get_thread_num();
        const int base = total / nth, extra = total % nth;
        count = base + (tid < extra ? 1 : 0);
        first = tid * base + (tid < extra ? tid : extra);
    }
#endif
    m_i = first;
    m_end = first + count;
}

inline Box MFIter::tilebox() const {
    const Box& v = m_mf->validBox();
    if (m_ts[1] == 0) return v;
    IntVect lo = v.smallEnd(), hi = v.bigEnd();
    int t = m_i;
    for (int d = 1; d < AMREX_SPACEDIM; ++d) {
        const int td = t % m_nt[d];
        t /= m_nt[d];
        lo[d] = v.smallEnd(d) + td * m_ts[d];
        hi[d] = std::min(lo[d] + m_ts[d] - 1, v.bigEnd(d));
    }
    return Box(lo, hi);
}
inline Box MFIter::validbox() const { return m_mf->validBox(); }
inline Box MFIter::fabbox() const { return m_mf->fab().box(); }

template <class F>
void ParallelFor(const Box& b, F&& f) {
    const int k0 = (AMREX_SPACEDIM == 3) ? b.smallEnd(2) : 0, k1 = (AMREX_SPACEDIM == 3) ? b.bigEnd(2) : 0;
    for (int k = k0; k <= k1; ++k)
        for (int j = b.smallEnd(1); j <= b.bigEnd(1); ++j)
            for (int i = b.smallEnd(0); i <= b.bigEnd(0); ++i) f(i, j, k);
}

template <class F>
void ParallelFor(const Box& b, int ncomp, F&& f) {
    for (int n = 0; n < ncomp; ++n) {
        const int k0 = (AMREX_SPACEDIM == 3) ? b.smallEnd(2) : 0, k1 = (AMREX_SPACEDIM == 3) ? b.bigEnd(2) : 0;
        for (int k = k0; k <= k1; ++k)
            for (int j = b.smallEnd(1); j <= b.bigEnd(1); ++j)
                for (int i = b.smallEnd(0); i <= b.bigEnd(0); ++i) f(i, j, k, n);
    }
}

namespace Gpu { inline void streamSynchronize() {} }

namespace BCType {
enum : int { int_dir = 0, reflect_odd = -1, reflect_even = 1, foextrap = 2, ext_dir = 3, hoextrap = 4,
             hoextrapcc = 5, user_1 = 1001 };
}

class BCRec {
public:
    void setLo(int d, int v) { m_lo[d] = v; }
    void setHi(int d, int v) { m_hi[d] = v; }
    int lo(int d) const { return m_lo[d]; }
    int hi(int d) const { return m_hi[d]; }
private:
    int m_lo[3] = {0, 0, 0}, m_hi[3] = {0, 0, 0};
};

struct GeometryData {
    Box domain;
    int is_periodic[3] = {0, 0, 0};
    const Box& Domain() const noexcept { return domain; }
    int isPeriodic(int d) const noexcept { return is_periodic[d]; }
};

class Geometry {
public:
    GeometryData data() const { return m_data; }
    const Box& Domain() const { return m_data.domain; }
    bool isPeriodic(int d) const { return m_data.is_periodic[d] != 0; }
    GeometryData m_data;
};

// Output is discarded: the checker only needs the numbers.
struct Print {
    template <class T> Print& operator<<(const T&) { return *this; }
    Print& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};

}  // namespace amrex

#endif
