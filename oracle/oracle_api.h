/* oracle_api.h -- C interface shared by the CPU oracle of the lattice-Boltzmann
 * step (lbm_oracle.cpp, a restatement of the reference algorithm) and by the
 * reference-kernel build under oracle/_ref/ (ref_driver.cpp compiled against
 * the reference's own LBM sources).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this; it is used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline arm as the checker.
 *
 * Layout conventions (mirroring the reference's AMReX FAB layout,
 * src/LBM/Collision.cpp:18-92 reads fin(i,j,k,n) with i fastest):
 *   - "valid" arrays: f[n][k][j][i], i fastest, n slowest, no ghost cells.
 *   - "ghost" arrays: the same with every spatial extent grown by one ghost
 *     layer (nGhost = 1, LatticeDescriptor.H:30); in 2-D there is no k ghost.
 *   - rho[k][j][i]; u[d][k][j][i] (velocity component slowest).
 * Face order is the reference's faceIndex(dir, bound) = 2*dir + (bound>0)
 * (BoundaryConditions.H:37-39): xlo, xhi, ylo, yhi, zlo, zhi.
 * BC type codes follow enum class lbmBCtype (BoundaryConditions.H:41):
 *   0 MovingWall, 1 NoSlip, 2 Inflow, 3 Outflow, 4 PressureOutlet, 5 Periodic.
 */
#ifndef MPH_ORACLE_API_H
#define MPH_ORACLE_API_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int dim;            /* 2 or 3 */
    int q;              /* 9 (dim 2); 15, 19, 27 (dim 3) */
    int n[3];           /* valid cells per direction; n[2] = 1 in 2-D */
    double omega;       /* BGK relaxation frequency 1/tau */
    int forced;         /* 1: Guo forcing path (SimulationImpl::m_has_forcing) */
    double F[3];        /* body force, lattice units */
    int face_type[6];   /* lbmBCtype per face; periodicity from the lo face */
    double face_rho[6]; /* face density, lattice units */
    double face_U[6][3];/* face velocity, lattice units */
} orc_desc;

typedef struct {
    int dim;
    int ncells[3];
    double prob_lo[3], prob_hi[3];
    double ref_length, ref_velocity, ref_density;
    int has_Re; double Re;
    int has_nu; double nu_phys;
    int has_u_lat; double u_lat;
    int has_tau; double tau;
} orc_units_in;

typedef struct {
    double dx, dt, u_lat, nu_lat, tau, omega, Re, nu_phys;
} orc_units_out;

/* UnitConverter (Units.cpp:20-183): derives the lattice scales and converts
 * nacc accelerations, nvel velocities and nrho densities from physical to
 * lattice units (toLatticeAcceleration / toLatticeVelocity /
 * toLatticeDensity).  Returns 0 on success, nonzero where the reference
 * would abort. */
int orc_units(const orc_units_in* in, orc_units_out* out,
              int nacc, const double* accel_phys, double* accel_lat,
              int nvel, const double* vel_phys, double* vel_lat,
              int nrho, const double* rho_phys, double* rho_lat);

/* Resolved 3^D ghost-class table (BCManager::finalize).  type/rho/U arrays of
 * length 27 (9 used in 2-D).  Returns nonzero on a conflicting edge/corner. */
int orc_resolve_bc(const orc_desc* d, int* type, double* rho, double* U /*27x3*/);

void* orc_create(const orc_desc* d);
void orc_destroy(void* s);
long long orc_ncells(void* s);
long long orc_nghost_cells(void* s);
int orc_set_f(void* s, const double* f);
int orc_get_f(void* s, double* f);
int orc_set_f_ghost(void* s, const double* f);
int orc_get_f_ghost(void* s, double* f);
/* FillBoundary(periodicity) followed by the physical BC ghost fill. */
int orc_fill_ghosts(void* s);
/* nsteps of SimulationImpl::advance(): pull-collide, swap, ghost fill. */
int orc_step(void* s, int nsteps, int nthreads);
/* SimulationImpl::setInitialConditions() from given (rho, u) followed by the
 * ghost fill of initialize(); rho/u are overwritten with the stored
 * macroscopic fields (changed only on the forced path). */
int orc_init_fields(void* s, double* rho, double* u);
/* SimulationImpl::updateMacroscopic(): stream, then moments. */
int orc_moments(void* s, double* rho, double* u);
/* Interior obstacles (no counterpart in the reference): mask[cell] != 0 marks
 * a solid cell (valid cells, x fastest); NULL removes them.  A population
 * whose upstream cell is solid takes the cell's own opposite population
 * (bounce-back with U = 0); solid cells hold f = w. */
int orc_set_obstacles(void* s, const unsigned char* mask);

#ifdef __cplusplus
}
#endif
#endif
