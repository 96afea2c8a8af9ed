// ref_driver.cpp -- drives the reference's own LBM sources (src/LBM/*.cpp of
// the reference project, compiled unchanged against the project-written AMReX
// stand-in in oracle/ref_shim/) behind the oracle C interface (oracle_api.h).
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into oracle/_ref/
// (one library per AMREX_SPACEDIM) on a host that has the reference sources;
// used to pin the CPU oracle (lbm_oracle.cpp) and to generate the golden
// fixtures under tests/golden/.
//
// What runs the reference's code: pullCollideFusedMF (Collision.cpp:95-143),
// BCManager<L>::operator() and finalize() (BoundaryConditions.H:124-189,
// BoundaryConditions.cpp:99-155), resolveBC / hasConflictingBC
// (BoundaryConditions.cpp:37-97), computeEquilibriumMF, initVelCorrection,
// computeMacroscopic, streamMF, UnitConverter.  What is restated here (AMReX
// itself is absent): the single-box FillBoundary periodic copy and the
// PhysBCFunct loop that calls BCManager on every ghost cell, i.e. the body of
// SimulationImpl::fillGhostCells (SimulationSetup.cpp:222-234), and the
// advance()/setInitialConditions()/updateMacroscopic() sequencing
// (SimulationSetup.cpp:120-219).
#include "oracle_api.h"

#include "LBM/BoundaryConditions.H"
#include "LBM/Collision.H"
#include "LBM/Equilibrium.H"
#include "LBM/LatticeDescriptor.H"
#include "LBM/Macroscopic.H"
#include "LBM/Streaming.H"
#include "LBM/Units.H"

#include <cstring>
#include <memory>
#include <optional>
#include <utility>

using namespace muphfasa;

namespace {

constexpr int D = AMREX_SPACEDIM;

struct Base {
    virtual ~Base() = default;
    virtual long long ncells() const = 0;
    virtual long long nghost() const = 0;
    virtual void setF(const double* f) = 0;
    virtual void getF(double* f) = 0;
    virtual void setFG(const double* f) = 0;
    virtual void getFG(double* f) = 0;
    virtual void fill() = 0;
    virtual void step(int n) = 0;
    virtual void init(double* rho, double* u) = 0;
    virtual void moments(double* rho, double* u) = 0;
};

template <class L>
struct Impl : Base {
    orc_desc d;
    amrex::Box dom;
    amrex::MultiFab fin, fout, rho, vel;
    amrex::Geometry geom;
    BCManager<L> bcm;
    amrex::BCRec bcr;
    amrex::GpuArray<amrex::Real, D> F{};

    explicit Impl(const orc_desc& dd) : d(dd) {
        dom = amrex::Box(amrex::IntVect(0), amrex::IntVect(AMREX_D_DECL(d.n[0] - 1, d.n[1] - 1, d.n[2] - 1)));
        fin.define(dom, L::Q, L::nGhost);
        fout.define(dom, L::Q, L::nGhost);
        rho.define(dom, 1, 0);
        vel.define(dom, D, 0);
        const double nan = std::nan("");
        fin.setVal(nan);
        fout.setVal(nan);
        geom.m_data.domain = dom;
        for (int dir = 0; dir < D; ++dir) {
            geom.m_data.is_periodic[dir] = (d.face_type[2 * dir] == (int)lbmBCtype::Periodic);
            F[dir] = d.F[dir];
        }
        // buildBCManager (SimulationSetup.cpp:237-299) with the face values
        // already in lattice units.
        for (int dir = 0; dir < D; ++dir) {
            for (int bound : {-1, 1}) {
                const int fi = faceIndex(dir, bound);
                if (d.face_type[fi] == (int)lbmBCtype::Periodic) {
                    AMREX_ALWAYS_ASSERT_WITH_MESSAGE(geom.isPeriodic(dir), "Periodic face on a non-periodic direction");
                    continue;
                }
                bcm.setFaceBC(dir, bound, (lbmBCtype)d.face_type[fi]);
                bcm.setFaceDensity(dir, bound, d.face_rho[fi]);
                amrex::GpuArray<amrex::Real, D> U{};
                for (int c = 0; c < D; ++c) U[c] = d.face_U[fi][c];
                bcm.setFaceVel(dir, bound, U);
            }
            bcr.setLo(dir, geom.isPeriodic(dir) ? amrex::BCType::int_dir : kCustomBCSentinel);
            bcr.setHi(dir, geom.isPeriodic(dir) ? amrex::BCType::int_dir : kCustomBCSentinel);
        }
        bcm.finalize();
    }

    long long ncells() const override { return (long long)d.n[0] * d.n[1] * d.n[2]; }
    long long nghost() const override { return (long long)fin.fab().const_array().nstride; }

    void setF(const double* f) override {
        auto a = fin.fab().array();
        long long c = 0;
        for (int n = 0; n < L::Q; ++n)
            amrex::ParallelFor(dom, [&](int i, int j, int k) { a(i, j, k, n) = f[c++]; });
    }
    void getF(double* f) override {
        auto a = fin.fab().const_array();
        long long c = 0;
        for (int n = 0; n < L::Q; ++n)
            amrex::ParallelFor(dom, [&](int i, int j, int k) { f[c++] = a(i, j, k, n); });
    }
    void setFG(const double* f) override {
        std::memcpy(fin.fab().data().data(), f, sizeof(double) * fin.fab().data().size());
    }
    void getFG(double* f) override {
        std::memcpy(f, fin.fab().data().data(), sizeof(double) * fin.fab().data().size());
    }

    // f(i, j, k) on every ghost cell of the ghost-grown box: whole rows
    // outside the domain in y or z, the row ends otherwise.  Rows are
    // independent (each pass reads valid cells only and writes its own ghost
    // cell), so they are shared among the OpenMP threads.
    template <class F>
    void for_each_ghost(const amrex::Box& gbox, F&& f) const {
        const int j0 = gbox.smallEnd(1), nj = gbox.length(1);
        const int k0 = D == 3 ? gbox.smallEnd(2) : 0, nk = D == 3 ? gbox.length(2) : 1;
        const long long rows = (long long)nj * nk;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long r = 0; r < rows; ++r) {
            const int j = j0 + (int)(r % nj), k = k0 + (int)(r / nj);
            const bool inside = j >= dom.smallEnd(1) && j <= dom.bigEnd(1) &&
                                (D == 2 || (k >= dom.smallEnd(D - 1) && k <= dom.bigEnd(D - 1)));
            for (int i = gbox.smallEnd(0); i <= gbox.bigEnd(0); ++i) {
                if (inside && i == dom.smallEnd(0)) i = dom.bigEnd(0) + 1;  // skip the valid run
                if (i > gbox.bigEnd(0)) break;
                f(i, j, k);
            }
        }
    }

    // fillGhostCells: FillBoundary(periodicity), then PhysBCFunct calling
    // BCManager on the ghost cells outside the domain.
    void fill() override {
        auto a = fin.fab().array();
        const amrex::Box gbox = fin.fab().box();
        for_each_ghost(gbox, [&](int i, int j, int k) {
            amrex::IntVect iv(AMREX_D_DECL(i, j, k));
            if (dom.contains(iv)) return;
            amrex::IntVect img = iv;
            for (int dir = 0; dir < D; ++dir) {
                if (iv[dir] < dom.smallEnd(dir) || iv[dir] > dom.bigEnd(dir)) {
                    if (!geom.isPeriodic(dir)) return;
                    img[dir] = (iv[dir] < dom.smallEnd(dir)) ? iv[dir] + dom.length(dir) : iv[dir] - dom.length(dir);
                }
            }
            for (int n = 0; n < L::Q; ++n) a(iv, n) = a(img, n);
        });
        const amrex::GeometryData gd = geom.data();
        for_each_ghost(gbox, [&](int i, int j, int k) {
            amrex::IntVect iv(AMREX_D_DECL(i, j, k));
            if (dom.contains(iv)) return;
            bcm(iv, a, 0, L::Q, gd, 0.0, &bcr, 0, 0);
        });
    }

    // SimulationImpl::advance, SimulationSetup.cpp:120-139.
    void step(int nsteps) override {
        for (int t = 0; t < nsteps; ++t) {
            if (d.forced) pullCollideFusedMF<L, BGK>(fin, fout, d.omega, F);
            else pullCollideFusedMF<L, BGK>(fin, fout, d.omega);
            std::swap(fin, fout);
            fill();
        }
    }

    void toMF(const double* r, const double* u) {
        auto ra = rho.fab().array();
        auto va = vel.fab().array();
        long long c = 0;
        amrex::ParallelFor(dom, [&](int i, int j, int k) { ra(i, j, k) = r[c++]; });
        for (int dd = 0; dd < D; ++dd) {
            c = 0;
            amrex::ParallelFor(dom, [&](int i, int j, int k) { va(i, j, k, dd) = u[dd * ncells() + c++]; });
        }
    }
    void fromMF(double* r, double* u) {
        auto ra = rho.fab().const_array();
        auto va = vel.fab().const_array();
        long long c = 0;
        amrex::ParallelFor(dom, [&](int i, int j, int k) { r[c++] = ra(i, j, k); });
        for (int dd = 0; dd < D; ++dd) {
            c = 0;
            amrex::ParallelFor(dom, [&](int i, int j, int k) { u[dd * ncells() + c++] = va(i, j, k, dd); });
        }
    }

    // setInitialConditions (SimulationSetup.cpp:201-219) + fillGhostCells.
    void init(double* r, double* u) override {
        toMF(r, u);
        if (!d.forced) {
            computeEquilibriumMF<L>(rho, vel, fin);
        } else {
            initVelCorrection(rho, vel, F);
            computeEquilibriumMF<L>(rho, vel, fin);
            computeMacroscopic<L>(fin, rho, vel, F);
        }
        fill();
        fromMF(r, u);
    }

    // updateMacroscopic (SimulationSetup.cpp:142-166).
    void moments(double* r, double* u) override {
        streamMF<L>(fin, fout, geom);
        if (!d.forced) computeMacroscopic<L>(fout, rho, vel);
        else computeMacroscopic<L>(fout, rho, vel, F);
        fromMF(r, u);
    }
};

Base* make(const orc_desc& d) {
#if (AMREX_SPACEDIM == 2)
    if (d.dim == 2 && d.q == 9) return new Impl<D2Q9>(d);
#else
    if (d.dim == 3 && d.q == 15) return new Impl<D3Q15>(d);
    if (d.dim == 3 && d.q == 19) return new Impl<D3Q19>(d);
    if (d.dim == 3 && d.q == 27) return new Impl<D3Q27>(d);
#endif
    return nullptr;
}

}  // namespace

extern "C" {

int orc_units(const orc_units_in* in, orc_units_out* out, int nacc, const double* accel_phys,
              double* accel_lat, int nvel, const double* vel_phys, double* vel_lat, int nrho,
              const double* rho_phys, double* rho_lat) {
    try {
        std::vector<int> N(D);
        std::vector<amrex::Real> lo(D), hi(D);
        for (int dd = 0; dd < D; ++dd) { N[dd] = in->ncells[dd]; lo[dd] = in->prob_lo[dd]; hi[dd] = in->prob_hi[dd]; }
        std::optional<amrex::Real> Re, nu, ul, tau;
        if (in->has_Re) Re = in->Re;
        if (in->has_nu) nu = in->nu_phys;
        if (in->has_u_lat) ul = in->u_lat;
        if (in->has_tau) tau = in->tau;
        UnitConverter uc(in->ref_length, in->ref_velocity, in->ref_density, N, lo, hi,
                         D2Q9::cs2, Re, nu, ul, tau);
        out->dx = uc.dx(); out->dt = uc.dt(); out->u_lat = uc.latticeVelocity();
        out->nu_lat = uc.latticeViscosity(); out->tau = uc.relaxationTime();
        out->omega = amrex::Real(1.0) / uc.relaxationTime();
        out->Re = uc.reynoldsNumber(); out->nu_phys = uc.physViscosity();
        for (int a = 0; a < nacc; ++a) accel_lat[a] = uc.toLatticeAcceleration(accel_phys[a]);
        for (int a = 0; a < nvel; ++a) vel_lat[a] = uc.toLatticeVelocity(vel_phys[a]);
        for (int a = 0; a < nrho; ++a) rho_lat[a] = uc.toLatticeDensity(rho_phys[a]);
        return 0;
    } catch (...) {
        return 1;
    }
}

// Enumerates the 3^D ghost classes the way BCManager::finalize does and lets
// the reference's resolveBC pick the winner (finalize's own table is private).
int orc_resolve_bc(const orc_desc* d, int* type, double* rho, double* U) {
    try {
        int total = 1;
        for (int dd = 0; dd < D; ++dd) total *= 3;
        for (int idx = 0; idx < 27; ++idx) {
            type[idx] = (int)lbmBCtype::Periodic; rho[idx] = 1.0;
            U[3 * idx] = U[3 * idx + 1] = U[3 * idx + 2] = 0.0;
        }
        for (int idx = 0; idx < total; ++idx) {
            int code[3] = {0, 0, 0}, tmp = idx;
            for (int dd = 0; dd < D; ++dd) { code[dd] = (tmp % 3) - 1; tmp /= 3; }
            amrex::Vector<lbmBCtype> types;
            amrex::Vector<amrex::Real> rhos;
            amrex::Vector<amrex::GpuArray<amrex::Real, D>> Us;
            amrex::Vector<std::string> names;
            for (int dd = 0; dd < D; ++dd) {
                if (code[dd] == 0) continue;
                const int fi = faceIndex(dd, code[dd]);
                if (d->face_type[fi] == (int)lbmBCtype::Periodic) continue;
                types.push_back((lbmBCtype)d->face_type[fi]);
                rhos.push_back(d->face_rho[fi]);
                amrex::GpuArray<amrex::Real, D> u{};
                for (int c = 0; c < D; ++c) u[c] = d->face_U[fi][c];
                Us.push_back(u);
                names.push_back("f");
            }
            if (types.empty()) continue;
            ResolvedFaceBC r = resolveBC(types, rhos, Us, names);
            type[idx] = (int)r.type;
            rho[idx] = r.rho;
            for (int c = 0; c < D; ++c) U[3 * idx + c] = r.U[c];
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

void* orc_create(const orc_desc* d) {
    try { return make(*d); } catch (...) { return nullptr; }
}
void orc_destroy(void* s) { delete static_cast<Base*>(s); }
long long orc_ncells(void* s) { return static_cast<Base*>(s)->ncells(); }
long long orc_nghost_cells(void* s) { return static_cast<Base*>(s)->nghost(); }
int orc_set_f(void* s, const double* f) { static_cast<Base*>(s)->setF(f); return 0; }
int orc_get_f(void* s, double* f) { static_cast<Base*>(s)->getF(f); return 0; }
int orc_set_f_ghost(void* s, const double* f) { static_cast<Base*>(s)->setFG(f); return 0; }
int orc_get_f_ghost(void* s, double* f) { static_cast<Base*>(s)->getFG(f); return 0; }
int orc_fill_ghosts(void* s) {
    try { static_cast<Base*>(s)->fill(); return 0; } catch (...) { return 1; }
}
// nthreads > 0 sets the OpenMP thread count of the reference's
// `#pragma omp parallel` MFIter loops (a build with -fopenmp).
int orc_step(void* s, int nsteps, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    try { static_cast<Base*>(s)->step(nsteps); return 0; } catch (...) { return 1; }
}
int orc_init_fields(void* s, double* rho, double* u) {
    try { static_cast<Base*>(s)->init(rho, u); return 0; } catch (...) { return 1; }
}
int orc_moments(void* s, double* rho, double* u) {
    try { static_cast<Base*>(s)->moments(rho, u); return 0; } catch (...) { return 1; }
}

}  // extern "C"
