// lbm_launch.h -- host-side launchers of the step kernels.  Each kernel
// translation unit defines the launchers of the precisions it compiles;
// sim.cu dispatches on the handle's precision.
#pragma once

#include <cuda_runtime.h>

#include "lbm_kernels.cuh"

namespace mph {

// Block of 256 threads with lanes along x (rows of one (y, z)), grid over
// (x-blocks, y-blocks, z).
// Step kernels cover the window rows [y0, y1) x planes [z0, z1) of KParams;
// other kernels (init, moments) are launched on the full domain only.
inline void step_shape(const KParams& p, dim3& grid, dim3& block, int threads = 256) {
    int bx = ((p.nx + 31) / 32) * 32;
    if (bx > threads) bx = threads;
    const int by = threads / bx;
    block = dim3(bx, by, 1);
    grid = dim3((p.nx + bx - 1) / bx, (p.y1 - p.y0 + by - 1) / by, p.z1 - p.z0);
}

// Plain 1-D shape over the cells.
inline void flat_shape(long long ncell, dim3& grid, dim3& block) {
    block = dim3(256, 1, 1);
    grid = dim3((unsigned)((ncell + 255) / 256), 1, 1);
}

// ---- k_f64_exact.cu (reference operation order, --fmad=false) ----------
cudaError_t launch_step_exact(int q, bool forced, const double* fin, double* fout, const KParams& p,
                              const KParams* pg, cudaStream_t s);
// prec selects the storage policy of fin (MPH_PREC_*); moments/init/reduce
// use the reference operation order in FP64 for every precision.
cudaError_t launch_moments(int prec, int q, bool forced, const void* fin, double* rho, double* u, const KParams& p,
                           const KParams* pg, cudaStream_t s);
cudaError_t launch_init(int prec, int q, bool forced, void* f, double* rho, double* u, const KParams& p,
                        cudaStream_t s);
cudaError_t launch_reduce(int prec, int q, const void* f, long long ncell, double* part, int nblocks, double* out4,
                          cudaStream_t s);
// f = feq + first-order non-equilibrium part from central differences of u
// (warm start, unforced domains).
cudaError_t launch_init_neq(int prec, int q, void* f, const double* rho, const double* u, const KParams& p,
                            cudaStream_t s);
// Uploads (to_store) OR 4 into *flag when a store saturates (weight-scaled
// 16-bit storage; flag may be null).
cudaError_t launch_convert(int prec, int q, bool to_store, void* store, double* f64, int n, long long ncell,
                           cudaStream_t s, int* flag = nullptr);
// All Q populations of the cells [c0, c0 + cnt) between the store and an FP64
// staging block laid out [q][cnt].
cudaError_t launch_convert_slab(int prec, int q, bool to_store, void* store, double* stage, long long c0,
                                long long cnt, long long ncell, cudaStream_t s, int* flag = nullptr);

struct A4 {
    double* p;
    long long js, ks, ns;
    int b[3], e[3];
};
cudaError_t launch_pull_collide_arr(int dim, int q, bool forced, const int lo[3], const int hi[3], const A4& fin,
                                    const A4& fout, const KParams& p, cudaStream_t s);
cudaError_t launch_periodic_fill_arr(int dim, int q, const int dlo[3], const int dhi[3], const int per[3],
                                     const A4& f, cudaStream_t s);
cudaError_t launch_bc_fill_arr(int dim, int q, const int dlo[3], const int dhi[3], const int per[3],
                               const KParams* pg, const A4& f, cudaStream_t s);

// ---- k_fast_*.cu (refactored FMA arithmetic) ----------------------------
cudaError_t launch_step_fast_f64(int q, bool forced, const double* fin, double* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s);
cudaError_t launch_step_fast_f32(int q, bool forced, const float* fin, float* fout, const KParams& p,
                                 const KParams* pg, cudaStream_t s);
cudaError_t launch_step_fast_f16s(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s);
cudaError_t launch_step_fast_bf16s(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                   const KParams* pg, cudaStream_t s);
cudaError_t launch_step_fast_f16c(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s);
cudaError_t launch_step_fast_f16w(int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, cudaStream_t s);
// The 16-bit pair step with bulk-copy staging (bulk_step.cuh): chunks of
// about `cells` cells of whole rows, `stages` shared-memory stages (2 or 3),
// total_elems = elements of the population array, flag |= 2 on a wait
// timeout.  mode 0 prepares the kernels (once per handle, before any launch
// or stream capture), mode 1 launches.  cudaErrorNotSupported when the launch
// does not apply (odd nx, obstacles, rows too long for shared memory): use
// the direct step then.
cudaError_t launch_step_bulk_f16s(int mode, int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, long long total_elems, int cells, int stages, int* flag,
                                  cudaStream_t s);
cudaError_t launch_step_bulk_bf16s(int mode, int q, bool forced, const void* fin, void* fout, const KParams& p,
                                   const KParams* pg, long long total_elems, int cells, int stages, int* flag,
                                   cudaStream_t s);
cudaError_t launch_step_bulk_f16c(int mode, int q, bool forced, const void* fin, void* fout, const KParams& p,
                                  const KParams* pg, long long total_elems, int cells, int stages, int* flag,
                                  cudaStream_t s);

// ---- k_f64x.cu (64-bit fixed point on the integer pipes) -----------------
cudaError_t launch_step_f64x(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                             const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                             cudaStream_t s);
// Persistent cp.async-pipelined variant; ctas = number of resident CTAs, as
// returned by f64x_pipe_ctas (which also raises the kernel's shared-memory
// limit, so it must run once before the first launch; 0 on error).
int f64x_pipe_ctas(int q, bool forced);
cudaError_t launch_step_f64x_pipe(int q, bool forced, const long long* fin, long long* fout, const KParams& p,
                                  const KParamsX& px, const KParams* pg, const long long* kbb, int* flag,
                                  int ctas, cudaStream_t s);

// ---- monitor.cu (steady-state residual, FP64) ---------------------------
// out2 = {sum |u - u_prev|^2, sum |u|^2} of the stored-population velocity;
// u_prev (dim x ncell doubles) is overwritten with u.
cudaError_t launch_residual(int prec, int q, const void* f, long long ncell, double* uprev, bool first, double* part,
                            int nblocks, double* out2, cudaStream_t s);

}  // namespace mph
