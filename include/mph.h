/* mph.h -- C ABI of the GB300-native lattice-Boltzmann time step.
 *
 * A drop-in for the stream-collide step of the reference solver (MuPhFASa):
 * the same inputs file, lattices (D2Q9, D3Q15, D3Q19, D3Q27), BGK relaxation,
 * Guo forcing and boundary types (NoSlip, MovingWall, Inflow, Outflow,
 * PressureOutlet, Periodic), computed by hand-written sm_103a CUDA kernels on
 * structure-of-arrays populations.
 *
 * Conventions
 *   - Every entry point returns an int status (MPH_OK on success) and never
 *     aborts the process; mph_last_error() gives the message of the calling
 *     thread's last failure.  Where the reference calls amrex::Abort the
 *     corresponding entry point returns MPH_ERR_CONFIG or MPH_ERR_PARSE.
 *   - Host population arrays are "valid-cell SoA": f[n][k][j][i], i fastest,
 *     population n slowest, exactly the component-last order of the
 *     reference's FABs without their ghost layer (Collision.cpp:18-92 reads
 *     fin(i,j,k,n)).  rho[k][j][i]; u[d][k][j][i].
 *   - Faces are ordered xlo, xhi, ylo, yhi, zlo, zhi (faceIndex,
 *     BoundaryConditions.H:37-39); a direction is periodic when its lo face is
 *     Periodic (GeometryHandler.cpp:39-48).
 *   - A simulation handle owns its device memory and one CUDA stream; calls
 *     on one handle are synchronous and not thread-safe; separate handles are
 *     independent.
 */
#ifndef MPH_H
#define MPH_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPH_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define MPH_OK 0
#define MPH_ERR_ARG 1          /* null pointer, bad size, bad enum value          */
#define MPH_ERR_CONFIG 2       /* configuration the reference rejects (aborts)    */
#define MPH_ERR_CUDA 3         /* CUDA runtime failure (message has the details)  */
#define MPH_ERR_UNSUPPORTED 4  /* recognised but not implemented (TRT/MRT, EB)    */
#define MPH_ERR_PARSE 5        /* inputs-file syntax, missing required key        */
#define MPH_ERR_NONFINITE 6    /* a checked step found NaN/Inf populations        */
#define MPH_ERR_STATE 7        /* call out of order (e.g. advance before init)    */

/* ---- boundary types: the order of enum class lbmBCtype
 *      (BoundaryConditions.H:41) ------------------------------------------- */
#define MPH_BC_MOVING_WALL 0
#define MPH_BC_NO_SLIP 1
#define MPH_BC_INFLOW 2
#define MPH_BC_OUTFLOW 3
#define MPH_BC_PRESSURE_OUTLET 4
#define MPH_BC_PERIODIC 5

/* ---- storage / arithmetic of the populations ---------------------------- */
/* FP64 storage, FP64 arithmetic in the reference's operation order: results
 * are bit-identical to the reference CPU path. */
#define MPH_PREC_F64 0
/* FP64 storage and arithmetic, FMA-contracted and refactored: agrees with the
 * reference to ~1e-15 per step (tested at 1e-12 after N steps). */
#define MPH_PREC_F64_FAST 1
/* FP32 storage and arithmetic. */
#define MPH_PREC_F32 2
/* f_i - w_i stored as FP16 / BF16, FP32 collide arithmetic. */
#define MPH_PREC_F16S 3
#define MPH_PREC_BF16S 4
/* 64-bit fixed-point storage of f_n / w_n (resolution 2^-56) with integer
 * arithmetic on the INT32/IMAD pipes: FP64-accurate (agrees with the reference
 * to ~1e-16 per step, tested at 1e-12 after N steps) at HBM speed on GB300,
 * whose FP64 pipes run at 1/64 of the FP32 rate.  Conversions to FP64 happen
 * only in mph_set_f / mph_get_f / moments / sums. */
#define MPH_PREC_F64X 5
/* f_i - w_i stored as a custom 16-bit float with one more significand bit
 * than FP16 (sign, 4 exponent bits biased by 16, 11 stored mantissa bits:
 * normals 2^-15 .. 1 - 2^-12, subnormal steps of 2^-26, larger magnitudes
 * saturate), FP32 collide arithmetic; same traffic as FP16 storage, half
 * its rounding error. */
#define MPH_PREC_F16C 6
/* (f_i - w_i) / p_i, p_i the power of two nearest to w_i, stored
 * as a custom 16-bit float (sign, 3 exponent bits biased by 8, 12 stored
 * mantissa bits: normals 2^-7 .. 1 - 2^-13, subnormal steps of 2^-19), FP32
 * collide arithmetic; same traffic as FP16 storage.  Scaling by about 1/w_i
 * puts every population's deviation on one scale, so the exponent needs one
 * bit less than MPH_PREC_F16C and the significand gets it.  Populations must
 * stay inside (w_i - p_i, w_i + p_i), p_i >= 0.75 w_i (|u| up to about 0.1):
 * a store that saturates (in a step, mph_set_f, mph_init_fields or
 * mph_init_fields_neq, and their batch forms) makes that call report
 * MPH_ERR_NONFINITE; the state is kept, saturated, and the steps go on
 * reporting it until a state within the range replaces it.  Single domains
 * and batches (the bulk-copy staged variants do not take it). */
#define MPH_PREC_F16W 7

/* ---- lattice-unit description of one domain ---------------------------- */
typedef struct {
    int dim;               /* 2 or 3                                          */
    int q;                 /* 9 (dim 2); 15, 19 or 27 (dim 3)                  */
    int n[3];              /* valid cells per direction; n[2] = 1 for dim 2    */
    double omega;          /* BGK relaxation frequency 1/tau                   */
    int forced;            /* 1 selects the Guo-forced kernels                 */
    double force[3];       /* body force, lattice units                        */
    int face_type[6];      /* MPH_BC_* per face                                */
    double face_rho[6];    /* face density (lattice units)                     */
    double face_U[6][3];   /* face velocity (lattice units)                    */
    int precision;         /* MPH_PREC_*                                       */
} mph_desc;

typedef struct {
    int type;              /* MPH_BC_* after edge/corner priority resolution   */
    double rho;
    double U[3];
} mph_resolved_bc;

/* Scales derived by the unit converter (Units.cpp:20-183) and the run
 * parameters of the driver loop (main.cpp:14-38, InputParser.cpp:92-323). */
typedef struct {
    double dx, dt, u_lat, nu_lat, tau, omega, Re, nu_phys;
    double ref_length, ref_velocity, ref_density;
    int max_step;
    double stop_time;      /* physical; <= 0 means run to max_step            */
    int plot_int, chk_int;
} mph_run_info;

const char* mph_last_error(void);
int mph_abi_version(void);
/* Page-locked host memory for the host-buffer calls (mph_step_host,
 * mph_set_f, mph_get_f): copies from it run at the full host link rate. */
int mph_host_alloc(long long bytes, void** out);
int mph_host_free(void* p);

/* Selects the CUDA device used by handles created afterwards on the calling
 * thread (the reference binds one device per MPI rank when AMReX initialises
 * its GPU backend; here one process drives one device). */
int mph_set_device(int device);

/* ---- inputs file: InputParser / UnitConverter / buildBCManager ----------- */
typedef struct mph_inputs mph_inputs;

/* Parses a ParmParse-style inputs file followed by "key=value" overrides
 * (amrex::Initialize(argc, argv); the last definition of a key wins).
 * path may be NULL to start from the overrides alone. */
int mph_inputs_load(const char* path, int noverrides, const char* const* overrides,
                    mph_inputs** out);
/* Same from an in-memory text. */
int mph_inputs_parse_string(const char* text, int noverrides, const char* const* overrides,
                            mph_inputs** out);
void mph_inputs_free(mph_inputs* in);
/* Raw value string of the last definition of `key` ("prefix.name");
 * MPH_ERR_ARG when absent. */
int mph_inputs_get(const mph_inputs* in, const char* key, char* buf, size_t buflen);
/* The lattice-unit domain description and scales that SimulationImpl's
 * constructor derives (SimulationSetup.cpp:32-89, 237-299). */
int mph_inputs_derive(const mph_inputs* in, int precision, mph_desc* desc, mph_run_info* info);

/* BCManager::finalize (BoundaryConditions.cpp:99-155): the 3^dim ghost-class
 * table indexed by sum_d (code_d + 1) 3^d.  table must hold 27 entries. */
int mph_resolve_bc(const mph_desc* desc, mph_resolved_bc* table);

/* ---- simulation handle: the ISimulation surface (ISimulation.H:16-44) ---- */
typedef struct mph_sim mph_sim;

int mph_create(const mph_desc* desc, mph_sim** out);
int mph_destroy(mph_sim* sim);
/* Upload / download populations (host valid-cell SoA, FP64). */
int mph_set_f(mph_sim* sim, const double* f);
int mph_get_f(mph_sim* sim, double* f);
/* setInitialConditions (SimulationSetup.cpp:201-219) from the given
 * macroscopic fields (what initData produces) plus the ghost fill of
 * initialize(); on the forced path rho/u are overwritten with the stored
 * macroscopic fields, as the reference overwrites m_rho/m_vel. */
int mph_init_fields(mph_sim* sim, double* rho, double* u);
/* nsteps x SimulationImpl::advance() (SimulationSetup.cpp:120-139).  With
 * MPH_PREC_F64X or MPH_PREC_F16W a state outside the storage's range makes
 * the call (and every later step call) return MPH_ERR_NONFINITE until the
 * state is replaced (mph_set_f, mph_init_fields, mph_init_fields_neq,
 * mph_set_state clear the handle's status). */
int mph_advance(mph_sim* sim, int nsteps);
/* updateMacroscopic (SimulationSetup.cpp:142-166): (rho, u) of the streamed,
 * pre-collision populations; u includes F/2 on the forced path. */
int mph_update_macroscopic(mph_sim* sim, double* rho, double* u);
/* FP64 sums of the stored populations: out[0] = sum f (mass),
 * out[1..3] = sum c f (momentum). */
int mph_reduce(mph_sim* sim, double* out);
/* Warm start (no counterpart in the reference): like mph_init_fields for an
 * unforced domain, plus the first-order Chapman-Enskog non-equilibrium part
 * f_neq_n = -(tau w_n rho / cs2)(c_n c_n - cs2 I) : grad u, grad u from
 * central differences of the given u (one-sided at non-periodic faces and
 * obstacles).  rho and u are not modified. */
int mph_init_fields_neq(mph_sim* sim, const double* rho, const double* u);
/* Interior obstacles (no counterpart in the reference; the reference's
 * embedded-boundary geometry is an unimplemented stub).  mask[cell] != 0
 * marks a solid cell (valid cells, x fastest); NULL removes all obstacles.
 * Rule: a population whose upstream cell x - c_n is solid takes the cell's
 * own opposite population (the BounceBack rule of BounceBack.H:36-63 with
 * U = 0 at the obstacle face); solid cells hold the rest state f = w.  Adds
 * one byte per cell of traffic.  Not available with MPH_F64X_KERNEL=pipe. */
int mph_set_obstacles(mph_sim* sim, const unsigned char* mask);
/* Steady-state residual (no counterpart in the reference), FP64 on the GPU:
 * with u = (sum c f) / (sum f) of the stored populations,
 *   out[0] = ||u - u_prev||_2 / ||u||_2, out[1] = ||u||_2,
 * where u_prev is the field saved by the previous call (out[0] = +inf on the
 * first call after a call that replaces the state: mph_create,
 * mph_init_fields, mph_init_fields_neq, mph_set_f, mph_set_state,
 * mph_step_host).  Calling it every k steps gives the relative change over
 * k steps. */
int mph_residual(mph_sim* sim, double* out);
/* Velocity set of a lattice (LatticeDescriptor.H:23-263): c[3 n + d],
 * w[n], opp[n] for n < q; any pointer may be NULL. */
int mph_lattice(int q, int* c, double* w, int* opp);
/* The populations in the handle's own storage format (FP64, FP32, shifted
 * 16-bit, or fixed-point int64; SoA, population slowest), for checkpoints
 * that resume bit for bit in every precision (the FP64 view of mph_get_f
 * rounds the 64-bit fixed point).  bytes must equal mph_state_bytes. */
int mph_state_bytes(const mph_sim* sim, long long* bytes);
int mph_get_state(mph_sim* sim, void* buf, long long bytes);
int mph_set_state(mph_sim* sim, const void* buf, long long bytes);
/* Sets the lattice time (a restart from a checkpoint, SimulationSetup.cpp:115). */
int mph_set_time(mph_sim* sim, double t);
/* Lattice time (number of completed advance() calls since init). */
int mph_time(const mph_sim* sim, double* t);
/* Number of step-kernel launches one advance() issues. */
int mph_launches_per_step(const mph_sim* sim, int* n);
/* nsteps advances timed with CUDA events on the handle's own stream;
 * *ms is the elapsed device time of the whole sequence. */
int mph_advance_timed(mph_sim* sim, int nsteps, float* ms);
/* Drop-in with host buffers: uploads f_in, advances nsteps, downloads the
 * result into f_out (both host valid-cell SoA FP64; may alias).  Domains of
 * 32 MB and more move in slabs of planes so that uploads, slab steps and
 * downloads overlap (MPH_STEP_HOST_SLABS sets the slab count, 0 disables);
 * the result is the same bits either way.  Page-locked buffers
 * (mph_host_alloc) reach the full host-link rate. */
int mph_step_host(mph_sim* sim, const double* f_in, double* f_out, int nsteps);

/* ---- plugin level: caller-owned device memory in AMReX Array4 layout ----- */
/* An Array4 view: element (i,j,k,n) lives at
 *   p[(i-begin[0]) + (j-begin[1])*jstride + (k-begin[2])*kstride + n*nstride]. */
typedef struct {
    double* p;
    long long jstride, kstride, nstride;
    int begin[3];
    int end[3];            /* exclusive */
    int ncomp;
} mph_array4;

/* pullCollideFusedArr<L,BGK> (Collision.cpp:18-92) over the cells
 * lo..hi (inclusive) of a ghost-grown fin; force NULL selects the unforced
 * variant.  Reference arithmetic order (bit-exact).  stream may be NULL. */
int mph_pull_collide_fused_arr(int dim, int q, const int lo[3], const int hi[3],
                               const mph_array4* fin, const mph_array4* fout, double omega,
                               const double* force, void* stream);
/* MultiFab::FillBoundary(periodicity) for one box covering the whole domain
 * dom_lo..dom_hi: ghost cells whose periodic image is valid receive all
 * components of that image (SimulationSetup.cpp:227). */
int mph_periodic_fill_arr(int dim, int q, const int dom_lo[3], const int dom_hi[3],
                          const int periodic[3], const mph_array4* f, void* stream);
/* BCManager<L>::operator() (BoundaryConditions.H:124-189) applied to every
 * ghost cell of f outside the domain, with the resolved table of
 * mph_resolve_bc. */
int mph_bc_fill_arr(int dim, int q, const int dom_lo[3], const int dom_hi[3],
                    const int periodic[3], const mph_resolved_bc* table, const mph_array4* f,
                    void* stream);

/* ---- batches of independent domains ------------------------------------ */
/* Many domains of uneven sizes advanced together (an ensemble of solver
 * instances; no counterpart API in the reference, which runs one domain per
 * process): one kernel per step covers every domain through a flat tile list,
 * step pairs are replayed from a CUDA graph, and the tile shape is chosen by
 * timing the candidates on the batch itself.  All domains share lattice,
 * precision (any MPH_PREC_*) and forcing flag; each has its own size,
 * omega, boundary faces and force.  Domain d's results equal those of a
 * single handle created from descs[d], bit for bit.  With MPH_PREC_F64X a
 * cell leaving the fixed-point range (with MPH_PREC_F16W a saturating store)
 * makes the advance return MPH_ERR_NONFINITE, as for a single handle, and
 * flags its domain (mph_batch_range_flags). */
typedef struct mph_batch mph_batch;
int mph_batch_create(int ndomains, const mph_desc* descs, mph_batch** out);
int mph_batch_destroy(mph_batch* b);
/* setInitialConditions of one domain (as mph_init_fields). */
int mph_batch_init_fields(mph_batch* b, int domain, double* rho, double* u);
int mph_batch_advance(mph_batch* b, int nsteps);
/* nsteps of the batched kernel timed with CUDA events (autotuning and graph
 * capture happen before the timed region). */
int mph_batch_advance_timed(mph_batch* b, int nsteps, float* ms);
/* The same steps as one single-domain launch per domain per step. */
int mph_batch_advance_looped_timed(mph_batch* b, int nsteps, float* ms);
int mph_batch_get_f(mph_batch* b, int domain, double* f);
/* Replaces one domain's populations (host valid-cell SoA FP64, converted to
 * the batch's storage), as mph_set_f for a single handle; the next
 * mph_batch_residual starts a new reference field for every domain. */
int mph_batch_set_f(mph_batch* b, int domain, const double* f);
int mph_batch_moments(mph_batch* b, int domain, double* rho, double* u);
/* Warm start of one batch domain, as mph_init_fields_neq. */
int mph_batch_init_fields_neq(mph_batch* b, int domain, const double* rho, const double* u);
/* Obstacles of one batch domain, as mph_set_obstacles. */
int mph_batch_set_obstacles(mph_batch* b, int domain, const unsigned char* mask);
/* Per-domain steady-state residual (as mph_residual): out[2 d] = relative
 * change of domain d's stored-population velocity since the previous call
 * (+inf on the first call after an init), out[2 d + 1] = ||u_d||_2. */
int mph_batch_residual(mph_batch* b, double* out);
/* Fixed-point and weight-scaled 16-bit batches (MPH_PREC_F64X,
 * MPH_PREC_F16W): flags[d] = 1 for every domain d whose populations left
 * the representable range in an advance since the domain was last
 * initialised or set (mph_batch_advance then returned
 * MPH_ERR_NONFINITE, and mph_batch_residual reports NaN for it).  The other
 * domains stepped normally: a caller can drop the flagged ones and go on.
 * All zero for other precisions.  No counterpart in the reference (its
 * single domain aborts on a non-finite density). */
int mph_batch_range_flags(const mph_batch* b, int* flags);
/* Total cells, cells per thread chosen by the autotuner (0 before the first
 * advance), the number of 256-thread chunks per step, and whether the chosen
 * launch is a persistent grid (1) or one block per chunk (0). */
int mph_batch_info(const mph_batch* b, long long* total_cells, int* cells_per_thread, int* nchunks, int* persistent);

/* ---- memory ceiling of the step ----------------------------------------- */
/* No counterpart in the reference.  Times the step's memory pattern without
 * its arithmetic on an nx x ny x nz periodic grid of q populations (q 9 with
 * nz = 1, or 19 / 27): every cell reads its populations from x - c_n and
 * writes them to its own slots, reps times (after two untimed passes), on
 * two buffers it allocates and frees.  elem_bytes 8, 4 or 2; mode 0 = one
 * cell per thread, 1 = cell pairs with 16-bit loads for x-shifted
 * populations (the 16-bit step kernel's pattern), 2 = cell pairs with one
 * aligned 32-bit word per population and warp shuffles for the x shift
 * (modes 1 and 2: 2-byte elements, nx even).  *ms = mean milliseconds per
 * pass; a pass moves 2 q elem_bytes bytes per cell. */
int mph_pull_copy_timed(int elem_bytes, int mode, int q, int nx, int ny, int nz, int reps, float* ms);
/* Instruction throughput of one arithmetic pipe of the current device
 * (operations per second, one per instruction), the rates that decide
 * which precision paths are compute-bound: op 0 DFMA, 1 FFMA, 2 32-bit
 * IMAD, 3 64-bit unsigned high multiply + add, 4 int64 -> FP64 conversion
 * + FP64 add.  No counterpart in the reference. */
int mph_pipe_rate(int op, double* ops_per_s);

/* ---- allocation-free sums ---------------------------------------------- */
/* No counterpart in the reference.  The FP64 mass and momentum sums of
 * mph_reduce, for callers that cannot allocate device memory (a solver inside
 * an application whose memory arena already holds the device, or one with a
 * no-allocation-after-start-up policy): f is caller-owned device memory in
 * valid-cell SoA layout (q * ncell doubles), out is caller-owned device
 * memory for 4 doubles (mass, momentum x, y, z), and the work is queued on
 * `stream` (NULL: the default stream) without synchronising.
 * The block partials live in a fixed 64 KiB device array inside the library
 * (held on every device that loads it until the process exits), which bounds
 * ncell at 134,217,728 (2048 slots x 65536 cells); larger sizes return
 * MPH_ERR_ARG.  No cudaMalloc/cudaFree or other allocating call is made.  The
 * first call on a device looks up the array's device address (once per
 * device), so that first call should come before any stream capture.  The
 * address stays cached for the life of the process: after cudaDeviceReset on
 * a device the library image is reloaded and the array may move, so do not
 * call this entry point on that device again in the same process.  Every
 * call shares the one array: calls that overlap on the GPU race and must be
 * ordered by the caller.  Nothing in the array needs to start at zero; every
 * slot a call reads is written earlier in the same call. */
int mph_reduce_f64_noalloc(int dim, int q, const double* f, long long ncell, double* out, void* stream);

/* ---- warm-start surrogate kernels ------------------------------------------
 * No counterpart in the reference.  Building blocks of the convolutional
 * neural operator that predicts steady (rho, u) fields (muphfasa_gb300/
 * surrogate.py drives them).  Activations are NHWC [P][C] (P = batch x H x W),
 * BF16 unless named float; a 3 x 3 conv's weights are Wt [Cout][9 Cin].  All
 * work is queued on `stream` (NULL = default stream); every call returns a
 * status code. */
int mph_nn_alloc(long long bytes, void** out);
int mph_nn_free(void* p);
/* dir: 0 host -> device, 1 device -> host (both synchronous), 2 device -> device. */
int mph_nn_copy(void* dst, const void* src, long long bytes, int dir, void* stream);
int mph_nn_sync(void* stream);
/* C (float, ldc) [+]= A . B on the tensor cores, BF16 operands, FP32
 * accumulation: A(m, k) = ta ? A[k lda + m] : A[m lda + k],
 * B(k, n) = tb ? B[k ldb + n] : B[n ldb + k].  GEMMs with few output tiles
 * split K into an FP32 workspace of the current device (a deterministic
 * reduce follows): calls on one device that may split must be ordered on
 * one stream.  (mph_nn_colsum keeps a per-device workspace the same way.) */
int mph_nn_gemm(int M, int N, int K, const void* A, long long lda, int ta, const void* B, long long ldb, int tb,
                float* C, long long ldc, int accumulate, void* stream);
/* GEMM kernel choice for later calls: 1 = mma.sync (m16n8k16) tiles, 2 =
 * tcgen05.mma with the accumulator in tensor memory (128 x 64 tiles, three
 * cp.async stages), 3 = the same single-buffered, 4 = tcgen05.mma fed by TMA
 * tensor copies (128 x 32/64/128 tiles, 64-wide K slices in 128-byte swizzled
 * layout, four stages; for ta = tb = 0 with 16-byte aligned bases and row
 * strides, mode 2 otherwise), 0 = automatic: mode 4 where it applies, else
 * mode 2, for M >= 128 or K >= 1024 with N >= 16, else mma.sync.  Not
 * thread-safe (process-wide setting). */
int mph_nn_gemm_mode(int mode);
/* Reads (and with reset != 0 clears) the flag the tcgen05 GEMM sets when a
 * bounded wait for its tensor-core work runs out. */
int mph_nn_status(int* timeout, int reset);
/* Y[p][co] (+)= 3 x 3, pad 1 convolution of the NHWC BF16 activation X
 * [Bn][H][W][C] with Wt [Cout][9 C] (tap-major, channel-minor): the GEMM of
 * im2col(X) with Wt^T without the im2col matrix (tcgen05 with TMA tensor
 * copies of each tap's shifted pixels, zero padding from TMA's out-of-range
 * fill).  MPH_ERR_UNSUPPORTED when C is not a multiple of 32 or image rows do
 * not tile into 128-pixel blocks (use mph_nn_im2col3 + mph_nn_gemm then). */
int mph_nn_conv3(const void* X, int Bn, int H, int W, int C, const void* Wt, int Cout, float* Y, int accumulate,
                 void* stream);
int mph_nn_im2col3(const void* X, int Bn, int H, int W, int C, void* Xcol, void* stream);
int mph_nn_col2im3(const float* dXcol, int Bn, int H, int W, int C, float* dX, void* stream);
/* out = act(Y + bias) into columns [c_off, c_off + C) of rows of width ld_out
 * (BF16 and/or float); act 1 = leaky ReLU (slope 0.1), 0 = identity. */
int mph_nn_bias_act(const float* Y, const float* bias, long long P, int C, int act, void* out_bf16, float* out_f32,
                    int ld_out, int c_off, void* stream);
int mph_nn_act_bwd(const float* dOut, int ld_dout, int c_off, const void* act_out, int ld_act, int act_off,
                   long long P, int C, int act, float* dPre, void* stream);
int mph_nn_colsum(const float* X, long long P, int C, float* out, void* stream);
int mph_nn_pool(const void* X, int Bn, int H, int W, int C, void* Y, void* stream);
int mph_nn_pool_bwd(const float* dY, int Bn, int H, int W, int C, float* dX, void* stream);
int mph_nn_up(const void* X, int Bn, int H, int W, int C, void* Y, int ldy, int c_off, void* stream);
int mph_nn_up_bwd(const float* dY, int ldy, int c_off, int Bn, int H, int W, int C, float* dX, void* stream);
/* Channel-slice copy; kind 0 BF16 -> BF16, 1 float -> float (optionally
 * accumulating), 2 float -> BF16. */
int mph_nn_slice(int kind, const void* src, int ld_src, int s_off, long long P, int C, void* dst, int ld_dst,
                 int d_off, int accumulate, void* stream);
/* Masked MSE: dpred = 2 w (pred - target) inv_count, part[b] = block sums of
 * w (pred - target)^2 (nblocks blocks of 256 threads). */
int mph_nn_mse(const float* pred, const float* target, const float* wgt, long long P, int C, float inv_count,
               float* dpred, float* part, int nblocks, void* stream);
/* Adam step t on FP32 masters with gradient grad * gscale and L2 decay wd. */
int mph_nn_adam(float* w, float* m, float* v, const float* grad, long long n, float lr, float b1, float b2, float eps,
                int t, float wd, float gscale, void* stream);
/* part[b] = block sums of x^2 (nblocks blocks of 256 threads). */
int mph_nn_sumsq(const float* x, long long n, float* part, int nblocks, void* stream);
/* kind 0 float -> BF16, 1 BF16 -> float. */
int mph_nn_cast(int kind, const void* x, long long n, void* y, void* stream);
int mph_nn_fill(float* x, long long n, float v, void* stream);
/* y[c][r] = x[r][c] for a rows x cols BF16 matrix (the K-contiguous layout
 * of a weight gradient's operands). */
int mph_nn_transpose(const void* x, long long rows, int cols, void* y, void* stream);
/* w2[ci][t cout + co] = wt[co][(8 - t) cin + ci] (BF16): the weights of a 3 x 3
 * convolution's data gradient as a convolution of dY with mirrored taps. */
int mph_nn_wflip(const void* wt, int cout, int cin, void* w2, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MPH_H */
