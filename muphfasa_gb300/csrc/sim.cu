// sim.cu -- the simulation handle behind the C ABI: device-resident
// populations (two SoA buffers swapped every step, the A/B pattern of
// SimulationImpl's m_fin/m_fout), one CUDA stream, and the ISimulation
// operations (ISimulation.H:16-44) mapped onto the kernels.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "lbm_launch.h"
#include "mph_internal.h"

using namespace mph;

struct mph_sim {
    mph_desc d;
    mph_resolved_bc table[27];
    KParams kp;
    KParamsX kpx;             // fixed-point constants (MPH_PREC_F64X)
    KParams* d_kp = nullptr;  // global copy for the boundary path
    long long* d_kbb = nullptr;  // fixed-point bounce-back constants [27][27]
    int* d_flag = nullptr;       // range flag of the fixed-point step (1), wait timeout of a staged step (2),
                                 // saturated weight-scaled 16-bit store (4)
    int pipe_ctas = 0;           // resident CTAs of the pipelined fixed-point kernel (0: direct kernel)
    int bulk_stages = 0;         // 16-bit storage: shared-memory stages of the bulk-copy step (0: direct kernel)
    int bulk_cells = 512;        // cells per chunk of the bulk-copy step
    size_t elem = 8;          // bytes per stored population value
    void* fa = nullptr;       // current populations (m_fin)
    void* fb = nullptr;       // next populations (m_fout)
    double* d_rho = nullptr;  // macroscopic scratch (init / moments)
    double* d_u = nullptr;
    double* d_stage = nullptr;  // FP64 staging of two populations (conversions)
    cudaStream_t copy_stream = nullptr;  // host copies overlapping the conversions
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_converted[2] = {nullptr, nullptr};
    // Slab pipeline of mph_step_host: uploads on copy_stream, upload
    // conversions and slab steps on stream, download conversions on
    // conv_stream, downloads on d2h_stream.
    static constexpr int kRing = 4;  // staging blocks per copy direction
    double* d_slab = nullptr;    // FP64 staging [2 kRing][q][slab_cells]: upload ring, download ring
    long long slab_cells = 0;    // cells of the largest slab
    long long max_pitch = 0;     // cudaDevAttrMaxPitch (row stride limit of 2-D copies)
    cudaStream_t d2h_stream = nullptr, conv_stream = nullptr;
    // up copied[kRing], up free[kRing], down converted[kRing], down free[kRing], start, stepped
    cudaEvent_t ev_slab[4 * kRing + 2] = {};
    double* d_part = nullptr;   // reduction partials
    double* d_red = nullptr;    // reduction result
    double* d_uprev = nullptr;  // velocity field saved by the last mph_residual (dim x N)
    unsigned char* d_cls = nullptr;  // obstacle class per cell (kp.cls), or null
    bool has_uprev = false;
    int red_blocks = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double time = 0.0;
    bool has_state = false;
    // Small domains: runs of graph_steps (even) steps replayed from a CUDA
    // graph, one per buffer the state starts in; 0 = plain launches.
    int graph_steps = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    void* graph_in[2] = {nullptr, nullptr};
};

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MPH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define MPH_CK(call, what)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, (what)); \
    } while (0)

size_t elem_size(int prec) {
    switch (prec) {
        case MPH_PREC_F64:
        case MPH_PREC_F64_FAST:
        case MPH_PREC_F64X: return 8;
        case MPH_PREC_F32: return 4;
        case MPH_PREC_F16S:
        case MPH_PREC_BF16S:
        case MPH_PREC_F16C:
        case MPH_PREC_F16W: return 2;
    }
    return 0;
}

template <int Q>
void guo_tables(const mph_desc& d, KParams& kp) {
    using L = Lat<Q>;
    for (int n = 0; n < 27; ++n) { kp.gpref[n] = 0.0; kp.gcF[n] = 0.0; }
    for (int n = 0; n < Q; ++n) {
        // guoForceTerm prefactor and c.F (Collision.H:21-65), same order.
        kp.gpref[n] = (1.0 - 0.5 * d.omega) * L::w(n) * 3.0;
        if (L::D == 2) kp.gcF[n] = L::cx(n) * kp.F[0] + L::cy(n) * kp.F[1];
        else kp.gcF[n] = L::cx(n) * kp.F[0] + L::cy(n) * kp.F[1] + L::cz(n) * kp.F[2];
    }
}

void build_params(const mph_desc& d, const mph_resolved_bc* tab, KParams& kp) {
    std::memset(&kp, 0, sizeof(kp));
    kp.nx = d.n[0];
    kp.ny = d.n[1];
    kp.nz = d.dim == 3 ? d.n[2] : 1;
    for (int a = 0; a < 3; ++a) kp.periodic[a] = (a < d.dim) && d.face_type[2 * a] == MPH_BC_PERIODIC;
    kp.ncell = (long long)kp.nx * kp.ny * kp.nz;
    kp.y1 = kp.ny;
    kp.z1 = kp.nz;
    kp.omega = d.omega;
    kp.omc = 1.0 - d.omega;
    for (int a = 0; a < 3; ++a) {
        kp.F[a] = (d.forced && a < d.dim) ? d.force[a] : 0.0;
        kp.hF[a] = 0.5 * kp.F[a];
    }
    switch (d.q) {
        case 9: guo_tables<9>(d, kp); break;
        case 15: guo_tables<15>(d, kp); break;
        case 19: guo_tables<19>(d, kp); break;
        case 27: guo_tables<27>(d, kp); break;
    }
    for (int c = 0; c < 27; ++c) {
        kp.bc_type[c] = tab[c].type;
        kp.bc_rho[c] = tab[c].rho;
        for (int a = 0; a < 3; ++a) kp.bc_U[c][a] = tab[c].U[a];
    }
    kp.omega_f = (float)kp.omega;
    kp.inv_nx_f = 1.0f / (float)kp.nx;
    kp.inv_ny_f = 1.0f / (float)kp.ny;
    for (int a = 0; a < 3; ++a) { kp.hF_f[a] = (float)kp.hF[a]; kp.F_f[a] = (float)kp.F[a]; }
    for (int n = 0; n < 27; ++n) { kp.gpref_f[n] = (float)kp.gpref[n]; kp.gcF_f[n] = (float)kp.gcF[n]; }
}

template <int Q>
void fixed_params(const mph_desc& d, const mph_resolved_bc* table, const KParams& kp, KParamsX& px, long long* kbb) {
    using L = Lat<Q>;
    std::memset(&px, 0, sizeof(px));
    px.W = (unsigned long long)std::ldexp(0.5 * d.omega, 64) & ~1ull;
    px.wh1 = (px.W >> 1) - 1;
    // 32 / iw_max, rounded to nearest (iw_max = 1 / smallest weight is an
    // integer: 36, 72, 36, 216).
    double iw_max = 0.0;
    for (int n = 0; n < Q; ++n) iw_max = L::iw(n) > iw_max ? L::iw(n) : iw_max;
    {
        const unsigned __int128 den = (unsigned __int128)iw_max;
        const unsigned __int128 num = (unsigned __int128)1 << 69;
        px.Wm = (unsigned long long)((num + den / 2) / den);
    }
    const double pre = 3.0 * (1.0 - 0.5 * d.omega) / d.omega;
    for (int a = 0; a < 3; ++a) {
        px.hF[a] = std::llrint(std::ldexp(kp.hF[a], 56));
        px.Fw[a] = std::llrint(std::ldexp(pre * kp.F[a], 56));
        if (px.Fw[a] != 0) px.fmask |= 1 << a;
    }
    // h-space bounce-back constants: contrib(opp n) / w_n with the
    // reference's contrib (BCTypes/BounceBack.H:56-63) evaluated in FP64.
    for (int c = 0; c < 27; ++c)
        for (int n = 0; n < 27; ++n) {
            kbb[c * 27 + n] = 0;
            const int t = table[c].type;
            if (n >= Q || !(t == MPH_BC_MOVING_WALL || t == MPH_BC_NO_SLIP || t == MPH_BC_INFLOW)) continue;
            const int o = L::opp(n);
            double rho = 1, U[3] = {0., 0., 0.};
            if (t != MPH_BC_NO_SLIP) {
                rho = table[c].rho;
                for (int a = 0; a < 3; ++a) U[a] = table[c].U[a];
            }
            double cdotu;
            if (L::D == 2) cdotu = L::cx(o) * U[0] + L::cy(o) * U[1];
            else cdotu = L::cx(o) * U[0] + L::cy(o) * U[1] + L::cz(o) * U[2];
            const double contrib = -2. * rho * L::w(o) * cdotu * 3.0;
            kbb[c * 27 + n] = std::llrint(std::ldexp(contrib * L::iw(n), 56));
        }
}

}  // namespace

namespace {
// Velocity set of lattice Q into plain arrays (mph_lattice).
template <int Q>
void lattice_tables(int* c, double* w, int* opp) {
    using L = Lat<Q>;
    for (int n = 0; n < Q; ++n) {
        if (c) { c[3 * n] = L::cx(n); c[3 * n + 1] = L::cy(n); c[3 * n + 2] = L::cz(n); }
        if (w) w[n] = L::w(n);
        if (opp) opp[n] = L::opp(n);
    }
}
}  // namespace

namespace {
// Class byte per cell from an obstacle mask: kSolid, kNearSolid (fluid with a
// solid upstream cell x - c_n, periodic images included, cells beyond a
// non-periodic face excluded) or kFluid.
template <int Q>
void classify(const KParams& p, const unsigned char* mask, unsigned char* cls) {
    using L = Lat<Q>;
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const long long c = ((long long)z * ny + y) * nx + x;
                if (mask[c]) { cls[c] = kSolid; continue; }
                unsigned char k = kFluid;
                for (int n = 1; n < Q && k == kFluid; ++n) {
                    int g[3] = {x - L::cx(n), y - L::cy(n), z - L::cz(n)};
                    const int dims[3] = {nx, ny, nz};
                    bool inside = true;
                    for (int a = 0; a < 3; ++a) {
                        if (g[a] >= 0 && g[a] < dims[a]) continue;
                        if (!p.periodic[a]) { inside = false; break; }
                        g[a] = g[a] < 0 ? g[a] + dims[a] : g[a] - dims[a];
                    }
                    if (inside && mask[((long long)g[2] * ny + g[1]) * nx + g[0]]) k = kNearSolid;
                }
                cls[c] = k;
            }
}
}  // namespace

namespace mph {
// ||u - u_prev|| / ||u|| from the two FP64 sums; NaN when the field is not
// finite (a diverged state never reads as converged), +inf before a previous
// field exists, 0 for a field that is zero and unchanged.
double relative_change(double s0, double s1, bool has_prev) {
    if (!std::isfinite(s0) || !std::isfinite(s1)) return std::nan("");
    if (!has_prev) return HUGE_VAL;
    if (s1 > 0.0) return std::sqrt(s0 / s1);
    return s0 > 0.0 ? HUGE_VAL : 0.0;
}

void build_cls(const KParams& p, int q, const unsigned char* mask, unsigned char* cls) {
    switch (q) {
        case 9: classify<9>(p, mask, cls); break;
        case 15: classify<15>(p, mask, cls); break;
        case 19: classify<19>(p, mask, cls); break;
        case 27: classify<27>(p, mask, cls); break;
    }
}
// KParams of one domain, shared with the batch (batch.cu).
void build_params_public(const mph_desc& d, const mph_resolved_bc* tab, KParams& kp) { build_params(d, tab, kp); }
// Fixed-point constants and the 27 x 27 bounce-back table of one domain
// (MPH_PREC_F64X), shared with the batch.
void build_fixed_public(const mph_desc& d, const mph_resolved_bc* tab, const KParams& kp, KParamsX& px,
                        long long* kbb) {
    switch (d.q) {
        case 9: fixed_params<9>(d, tab, kp, px, kbb); break;
        case 15: fixed_params<15>(d, tab, kp, px, kbb); break;
        case 19: fixed_params<19>(d, tab, kp, px, kbb); break;
        case 27: fixed_params<27>(d, tab, kp, px, kbb); break;
    }
}
}  // namespace mph

namespace {

void free_all(mph_sim* s) {
    if (!s) return;
    cudaFree(s->fa);
    cudaFree(s->fb);
    cudaFree(s->d_kp);
    cudaFree(s->d_kbb);
    cudaFree(s->d_flag);
    cudaFree(s->d_rho);
    cudaFree(s->d_u);
    cudaFree(s->d_stage);
    cudaFree(s->d_part);
    cudaFree(s->d_red);
    cudaFree(s->d_uprev);
    cudaFree(s->d_cls);
    for (cudaGraphExec_t g : s->graph)
        if (g) cudaGraphExecDestroy(g);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    for (int i = 0; i < 2; ++i) {
        if (s->ev_copied[i]) cudaEventDestroy(s->ev_copied[i]);
        if (s->ev_converted[i]) cudaEventDestroy(s->ev_converted[i]);
    }
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    cudaFree(s->d_slab);
    for (cudaEvent_t e : s->ev_slab)
        if (e) cudaEventDestroy(e);
    if (s->d2h_stream) cudaStreamDestroy(s->d2h_stream);
    if (s->conv_stream) cudaStreamDestroy(s->conv_stream);
    if (s->stream) cudaStreamDestroy(s->stream);
}

int ensure_macro(mph_sim* s) {
    if (!s->d_rho) MPH_CK(cudaMalloc(&s->d_rho, sizeof(double) * s->kp.ncell), "cudaMalloc(rho)");
    if (!s->d_u) MPH_CK(cudaMalloc(&s->d_u, sizeof(double) * 3 * s->kp.ncell), "cudaMalloc(u)");
    return MPH_OK;
}

int ensure_copy_stream(mph_sim* s) {
    if (!s->copy_stream) {
        MPH_CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "copy stream");
        for (int i = 0; i < 2; ++i) {
            MPH_CK(cudaEventCreateWithFlags(&s->ev_copied[i], cudaEventDisableTiming), "copy event");
            MPH_CK(cudaEventCreateWithFlags(&s->ev_converted[i], cudaEventDisableTiming), "copy event");
        }
    }
    return MPH_OK;
}

int ensure_stage(mph_sim* s) {
    if (!s->d_stage) MPH_CK(cudaMalloc(&s->d_stage, 2 * sizeof(double) * s->kp.ncell), "cudaMalloc(stage)");
    return ensure_copy_stream(s);
}

bool is_f64(const mph_sim* s) { return s->d.precision == MPH_PREC_F64 || s->d.precision == MPH_PREC_F64_FAST; }

// The bulk-copy staged step of the 16-bit storages (mode 0: prepare the
// kernel once, mode 1: one step fa -> fb over the window of kp).
cudaError_t launch_bulk(mph_sim* s, int mode, const KParams& kp) {
    const long long total = (long long)s->d.q * s->kp.ncell;
    const int q = s->d.q, st = s->bulk_stages, cells = s->bulk_cells;
    const bool forced = s->d.forced != 0;
    switch (s->d.precision) {
        case MPH_PREC_F16S:
            return launch_step_bulk_f16s(mode, q, forced, s->fa, s->fb, kp, s->d_kp, total, cells, st, s->d_flag, s->stream);
        case MPH_PREC_BF16S:
            return launch_step_bulk_bf16s(mode, q, forced, s->fa, s->fb, kp, s->d_kp, total, cells, st, s->d_flag, s->stream);
        case MPH_PREC_F16C:
            return launch_step_bulk_f16c(mode, q, forced, s->fa, s->fb, kp, s->d_kp, total, cells, st, s->d_flag, s->stream);
    }
    return cudaErrorNotSupported;
}

// One step fa -> fb over the window of kp (the whole domain, or a slab of
// planes for the host-copy pipeline; slabs take the direct fixed-point kernel).
cudaError_t launch_step_window(mph_sim* s, const KParams& kp, bool whole) {
    const int q = s->d.q;
    const bool forced = s->d.forced != 0;
    switch (s->d.precision) {
        case MPH_PREC_F64:
            return launch_step_exact(q, forced, (const double*)s->fa, (double*)s->fb, kp, s->d_kp, s->stream);
        case MPH_PREC_F64_FAST:
            return launch_step_fast_f64(q, forced, (const double*)s->fa, (double*)s->fb, kp, s->d_kp, s->stream);
        case MPH_PREC_F32:
            return launch_step_fast_f32(q, forced, (const float*)s->fa, (float*)s->fb, kp, s->d_kp, s->stream);
        case MPH_PREC_F16S:
        case MPH_PREC_BF16S:
        case MPH_PREC_F16C: {
            if (s->bulk_stages > 0) {
                const cudaError_t e = launch_bulk(s, 1, kp);
                if (e != cudaErrorNotSupported) return e;
            }
            if (s->d.precision == MPH_PREC_F16S)
                return launch_step_fast_f16s(q, forced, s->fa, s->fb, kp, s->d_kp, s->stream);
            if (s->d.precision == MPH_PREC_BF16S)
                return launch_step_fast_bf16s(q, forced, s->fa, s->fb, kp, s->d_kp, s->stream);
            return launch_step_fast_f16c(q, forced, s->fa, s->fb, kp, s->d_kp, s->stream);
        }
        case MPH_PREC_F16W:
            return launch_step_fast_f16w(q, forced, s->fa, s->fb, kp, s->d_kp, s->stream);
        case MPH_PREC_F64X:
            if (whole && s->pipe_ctas > 0)
                return launch_step_f64x_pipe(q, forced, (const long long*)s->fa, (long long*)s->fb, kp, s->kpx,
                                             s->d_kp, s->d_kbb, s->d_flag, s->pipe_ctas, s->stream);
            return launch_step_f64x(q, forced, (const long long*)s->fa, (long long*)s->fb, kp, s->kpx, s->d_kp,
                                    s->d_kbb, s->d_flag, s->stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_one_step(mph_sim* s) { return launch_step_window(s, s->kp, true); }

// Status flag: a cell of the fixed-point step left the representable range
// (1), a wait of a staged step timed out (2), a weight-scaled 16-bit store
// saturated (4).
int check_flag(mph_sim* s) {
    if (s->d.precision != MPH_PREC_F64X && s->d.precision != MPH_PREC_F16W && s->bulk_stages == 0) return MPH_OK;
    int flag = 0;
    MPH_CK(cudaMemcpyAsync(&flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "read flag");
    MPH_CK(cudaStreamSynchronize(s->stream), "read flag");
    if (flag & 2) {
        MPH_CK(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream), "clear flag");
        return fail(MPH_ERR_CUDA, "staged 16-bit step: a wait for bulk-copied operands exceeded its time limit "
                                  "(the step's results are incomplete)");
    }
    if (flag & 4) return fail(MPH_ERR_NONFINITE, "weight-scaled 16-bit storage: a population deviation "
                                                   "|f - w| reached the format's range p (p the power of two "
                                                   "nearest to w) and saturated, or was not finite");
    if (flag) return fail(MPH_ERR_NONFINITE, "fixed-point step: a cell left the representable range "
                                               "(rho outside (1/16, 64) or |J|, |u| >= 4)");
    return MPH_OK;
}

void drop_graphs(mph_sim* s) {
    for (int i = 0; i < 2; ++i) {
        if (s->graph[i]) cudaGraphExecDestroy(s->graph[i]);
        s->graph[i] = nullptr;
        s->graph_in[i] = nullptr;
    }
}

// graph_steps steps captured for each buffer the state can start in
// (A -> B -> ... -> A and B -> A -> ... -> B); the captured launches carry
// the parameters of the handle as they are now, so anything that changes
// them (obstacles) drops the graphs.
int ensure_graphs(mph_sim* s) {
    if (s->graph[0] && s->graph[1]) return MPH_OK;
    drop_graphs(s);
    void* const fa0 = s->fa;
    void* const fb0 = s->fb;
    for (int i = 0; i < 2; ++i) {
        s->fa = i == 0 ? fa0 : fb0;
        s->fb = i == 0 ? fb0 : fa0;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int t = 0; t < s->graph_steps && e == cudaSuccess; ++t) {
                e = launch_one_step(s);
                std::swap(s->fa, s->fb);
            }
            const cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&s->graph[i], g, 0);
        if (g) cudaGraphDestroy(g);
        s->graph_in[i] = i == 0 ? fa0 : fb0;
        s->fa = fa0;
        s->fb = fb0;
        if (e != cudaSuccess) {
            drop_graphs(s);
            return cuda_fail(e, "step graph capture");
        }
    }
    return MPH_OK;
}

int advance_async(mph_sim* s, int nsteps) {
    if (s->graph_steps > 0 && nsteps >= s->graph_steps) {
        int rc = ensure_graphs(s);
        if (rc) return rc;
        // an even run leaves the state in the buffer it started from
        const cudaGraphExec_t g = s->fa == s->graph_in[0] ? s->graph[0] : s->graph[1];
        for (; nsteps >= s->graph_steps; nsteps -= s->graph_steps) {
            MPH_CK(cudaGraphLaunch(g, s->stream), "step graph launch");
            s->time += s->graph_steps;  // SimulationSetup.cpp:138, per step
        }
    }
    for (int t = 0; t < nsteps; ++t) {
        cudaError_t e = launch_one_step(s);
        if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
        std::swap(s->fa, s->fb);  // SimulationSetup.cpp:132
    }
    s->time += nsteps;  // SimulationSetup.cpp:138
    return MPH_OK;
}

int upload(mph_sim* s, const double* f) {
    const size_t n = (size_t)s->d.q * s->kp.ncell;
    if (is_f64(s)) {
        MPH_CK(cudaMemcpyAsync(s->fa, f, n * sizeof(double), cudaMemcpyHostToDevice, s->stream), "upload f");
        return MPH_OK;
    }
    int rc = ensure_stage(s);
    if (rc) return rc;
    // Double-buffered: the copy of population q into stage q % 2 (copy
    // stream) overlaps the conversion of population q - 1 (handle stream).
    const size_t N = (size_t)s->kp.ncell;
    MPH_CK(cudaEventRecord(s->ev_converted[0], s->stream), "upload order");
    MPH_CK(cudaEventRecord(s->ev_converted[1], s->stream), "upload order");
    for (int q = 0; q < s->d.q; ++q) {
        const int b = q & 1;
        double* st = s->d_stage + b * N;
        MPH_CK(cudaStreamWaitEvent(s->copy_stream, s->ev_converted[b], 0), "upload order");
        MPH_CK(cudaMemcpyAsync(st, f + (size_t)q * N, sizeof(double) * N, cudaMemcpyHostToDevice, s->copy_stream),
               "upload f");
        MPH_CK(cudaEventRecord(s->ev_copied[b], s->copy_stream), "upload order");
        MPH_CK(cudaStreamWaitEvent(s->stream, s->ev_copied[b], 0), "upload order");
        MPH_CK(launch_convert(s->d.precision, s->d.q, true, s->fa, st, q, s->kp.ncell, s->stream, s->d_flag),
               "convert f");
        MPH_CK(cudaEventRecord(s->ev_converted[b], s->stream), "upload order");
    }
    return MPH_OK;
}

int download(mph_sim* s, double* f) {
    const size_t n = (size_t)s->d.q * s->kp.ncell;
    if (is_f64(s)) {
        MPH_CK(cudaMemcpyAsync(f, s->fa, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream), "download f");
        return MPH_OK;
    }
    int rc = ensure_stage(s);
    if (rc) return rc;
    // Double-buffered: the conversion of population q (handle stream)
    // overlaps the copy of population q - 1 to the host (copy stream); the
    // handle stream waits for the last copy, so sync() covers everything.
    const size_t N = (size_t)s->kp.ncell;
    MPH_CK(cudaEventRecord(s->ev_copied[0], s->copy_stream), "download order");
    MPH_CK(cudaEventRecord(s->ev_copied[1], s->copy_stream), "download order");
    for (int q = 0; q < s->d.q; ++q) {
        const int b = q & 1;
        double* st = s->d_stage + b * N;
        MPH_CK(cudaStreamWaitEvent(s->stream, s->ev_copied[b], 0), "download order");
        MPH_CK(launch_convert(s->d.precision, s->d.q, false, s->fa, st, q, s->kp.ncell, s->stream), "convert f");
        MPH_CK(cudaEventRecord(s->ev_converted[b], s->stream), "download order");
        MPH_CK(cudaStreamWaitEvent(s->copy_stream, s->ev_converted[b], 0), "download order");
        MPH_CK(cudaMemcpyAsync(f + (size_t)q * N, st, sizeof(double) * N, cudaMemcpyDeviceToHost, s->copy_stream),
               "download f");
        MPH_CK(cudaEventRecord(s->ev_copied[b], s->copy_stream), "download order");
    }
    MPH_CK(cudaStreamWaitEvent(s->stream, s->ev_copied[(s->d.q - 1) & 1], 0), "download order");
    return MPH_OK;
}

// ---- host-copy pipeline of mph_step_host ------------------------------
// The domain is cut into S slabs of whole planes of its outermost axis (z in
// 3-D, y in 2-D); a slab's populations are q contiguous runs of the SoA
// arrays.  Uploads run in the order S-1, 0, 1, ..., S-2 on copy_stream; slab
// k steps once slabs k-1, k, k+1 are resident (the pull reaches one plane),
// and its result goes back on d2h_stream while later slabs still upload, so
// the two copy directions overlap each other and the kernels.  Download
// conversions run on their own stream: a download waiting for a free staging
// block never holds up the uploads.  Slabs touch disjoint host ranges, so
// f_in may alias f_out.
// MPH_STEP_HOST_SLABS overrides the slab count (0: one block copy each way).
int slab_count(const mph_sim* s) {
    const int E = s->d.dim == 3 ? s->kp.nz : s->kp.ny;
    int S = 64;
    if (const char* env = std::getenv("MPH_STEP_HOST_SLABS")) {
        S = std::atoi(env);
        if (S <= 0) return 0;
    } else if ((long long)s->d.q * s->kp.ncell * 8 < (32LL << 20)) {
        return 0;  // small: one block copy
    }
    if (E < 3 || S < 3) return 0;
    return E < S ? E : S;
}

void slab_window(const mph_sim* s, int k, int S, KParams& w, long long& c0, long long& cnt) {
    const bool d3 = s->d.dim == 3;
    const int E = d3 ? s->kp.nz : s->kp.ny;
    const long long plane = d3 ? (long long)s->kp.nx * s->kp.ny : s->kp.nx;
    const int a = (int)((long long)k * E / S), b = (int)((long long)(k + 1) * E / S);
    w = s->kp;
    if (d3) { w.z0 = a; w.z1 = b; }
    else { w.y0 = a; w.y1 = b; }
    c0 = a * plane;
    cnt = (b - a) * plane;
}

int ensure_slabs(mph_sim* s, int S) {
    int rc = ensure_copy_stream(s);
    if (rc) return rc;
    if (!s->d2h_stream) {
        MPH_CK(cudaStreamCreateWithFlags(&s->d2h_stream, cudaStreamNonBlocking), "d2h stream");
        MPH_CK(cudaStreamCreateWithFlags(&s->conv_stream, cudaStreamNonBlocking), "conversion stream");
        for (cudaEvent_t& e : s->ev_slab) MPH_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "slab event");
        int dev = 0, pitch = 0;
        MPH_CK(cudaGetDevice(&dev), "cudaGetDevice");
        MPH_CK(cudaDeviceGetAttribute(&pitch, cudaDevAttrMaxPitch, dev), "max pitch");
        s->max_pitch = pitch;
    }
    const int E = s->d.dim == 3 ? s->kp.nz : s->kp.ny;
    const long long plane = s->kp.ncell / E;
    const long long cells = ((E + S - 1) / S) * plane;
    if (!is_f64(s) && cells > s->slab_cells) {
        cudaFree(s->d_slab);
        s->d_slab = nullptr;
        s->slab_cells = 0;
        MPH_CK(cudaMalloc(&s->d_slab, 2 * mph_sim::kRing * sizeof(double) * s->d.q * cells),
               "cudaMalloc(slab stage)");
        s->slab_cells = cells;
    }
    return MPH_OK;
}

// q rows of cnt values with the given row strides (elements): one 2-D copy,
// or one copy per row when a stride exceeds the 2-D pitch limit.
int copy_rows(const mph_sim* s, double* dst, long long dstride, const double* src, long long sstride, long long cnt,
              cudaMemcpyKind kind, cudaStream_t st) {
    const long long dp = dstride * (long long)sizeof(double), sp = sstride * (long long)sizeof(double);
    if (dp <= s->max_pitch && sp <= s->max_pitch) {
        MPH_CK(cudaMemcpy2DAsync(dst, (size_t)dp, src, (size_t)sp, sizeof(double) * cnt, (size_t)s->d.q, kind, st),
               "slab copy");
        return MPH_OK;
    }
    for (int n = 0; n < s->d.q; ++n)
        MPH_CK(cudaMemcpyAsync(dst + n * dstride, src + n * sstride, sizeof(double) * cnt, kind, st), "slab copy");
    return MPH_OK;
}

int slab_up(mph_sim* s, const double* f, int k, int S, int b) {
    KParams w;
    long long c0, cnt;
    slab_window(s, k, S, w, c0, cnt);
    const long long N = s->kp.ncell;
    constexpr int R = mph_sim::kRing;
    cudaEvent_t copied = s->ev_slab[b], freed = s->ev_slab[R + b];
    int rc;
    if (is_f64(s)) {
        if ((rc = copy_rows(s, (double*)s->fa + c0, N, f + c0, N, cnt, cudaMemcpyHostToDevice, s->copy_stream)))
            return rc;
        MPH_CK(cudaEventRecord(copied, s->copy_stream), "upload order");
        MPH_CK(cudaStreamWaitEvent(s->stream, copied, 0), "upload order");
        return MPH_OK;
    }
    double* st = s->d_slab + (size_t)b * s->d.q * s->slab_cells;
    MPH_CK(cudaStreamWaitEvent(s->copy_stream, freed, 0), "upload order");
    if ((rc = copy_rows(s, st, cnt, f + c0, N, cnt, cudaMemcpyHostToDevice, s->copy_stream))) return rc;
    MPH_CK(cudaEventRecord(copied, s->copy_stream), "upload order");
    MPH_CK(cudaStreamWaitEvent(s->stream, copied, 0), "upload order");
    MPH_CK(launch_convert_slab(s->d.precision, s->d.q, true, s->fa, st, c0, cnt, N, s->stream, s->d_flag),
           "convert slab");
    MPH_CK(cudaEventRecord(freed, s->stream), "upload order");
    return MPH_OK;
}

// Result of slab k, in fb, to the host.
int slab_down(mph_sim* s, double* f, int k, int S, int b) {
    KParams w;
    long long c0, cnt;
    slab_window(s, k, S, w, c0, cnt);
    const long long N = s->kp.ncell;
    constexpr int R = mph_sim::kRing;
    cudaEvent_t converted = s->ev_slab[2 * R + b], freed = s->ev_slab[3 * R + b], stepped = s->ev_slab[4 * R + 1];
    if (is_f64(s)) {
        MPH_CK(cudaEventRecord(stepped, s->stream), "download order");
        MPH_CK(cudaStreamWaitEvent(s->d2h_stream, stepped, 0), "download order");
        int rc = copy_rows(s, f + c0, N, (const double*)s->fb + c0, N, cnt, cudaMemcpyDeviceToHost, s->d2h_stream);
        if (rc) return rc;
        MPH_CK(cudaEventRecord(freed, s->d2h_stream), "download order");
        return MPH_OK;
    }
    double* st = s->d_slab + (size_t)(R + b) * s->d.q * s->slab_cells;
    MPH_CK(cudaEventRecord(stepped, s->stream), "download order");
    MPH_CK(cudaStreamWaitEvent(s->conv_stream, stepped, 0), "download order");
    MPH_CK(cudaStreamWaitEvent(s->conv_stream, freed, 0), "download order");
    MPH_CK(launch_convert_slab(s->d.precision, s->d.q, false, s->fb, st, c0, cnt, N, s->conv_stream),
           "convert slab");
    MPH_CK(cudaEventRecord(converted, s->conv_stream), "download order");
    MPH_CK(cudaStreamWaitEvent(s->d2h_stream, converted, 0), "download order");
    int rc = copy_rows(s, f + c0, N, st, cnt, cnt, cudaMemcpyDeviceToHost, s->d2h_stream);
    if (rc) return rc;
    MPH_CK(cudaEventRecord(freed, s->d2h_stream), "download order");
    return MPH_OK;
}

int slab_step(mph_sim* s, int k, int S) {
    KParams w;
    long long c0, cnt;
    slab_window(s, k, S, w, c0, cnt);
    MPH_CK(launch_step_window(s, w, false), "slab step launch");
    return MPH_OK;
}

// mph_step_host with nsteps >= 1 over S >= 3 slabs: the first step runs slab
// by slab behind the uploads, the last slab by slab ahead of the downloads.
int step_host_slabs(mph_sim* s, const double* f_in, double* f_out, int nsteps, int S) {
    int rc = ensure_slabs(s, S);
    if (rc) return rc;
    constexpr int R = mph_sim::kRing;
    cudaEvent_t start = s->ev_slab[4 * R];
    // Earlier work on the handle's stream comes first; every staging block starts free.
    MPH_CK(cudaEventRecord(start, s->stream), "pipeline order");
    MPH_CK(cudaStreamWaitEvent(s->copy_stream, start, 0), "pipeline order");
    MPH_CK(cudaStreamWaitEvent(s->d2h_stream, start, 0), "pipeline order");
    for (int b = 0; b < R; ++b) {
        MPH_CK(cudaEventRecord(s->ev_slab[R + b], s->stream), "pipeline order");
        MPH_CK(cudaEventRecord(s->ev_slab[3 * R + b], s->d2h_stream), "pipeline order");
    }
    const bool one = nsteps == 1;
    int nd = 0;  // downloads issued (staging block nd % R)
    auto step_and_send = [&](int k) {
        int r = slab_step(s, k, S);
        if (!r && one) r = slab_down(s, f_out, k, S, nd++ % R);
        return r;
    };
    // Step 1 behind the uploads S-1, 0, 1, ..., S-2.
    for (int i = 0; i < S; ++i) {
        const int k = i == 0 ? S - 1 : i - 1;
        if ((rc = slab_up(s, f_in, k, S, i % R))) return rc;
        if (i >= 2 && (rc = step_and_send(i - 2))) return rc;
    }
    if ((rc = step_and_send(S - 2)) || (rc = step_and_send(S - 1))) return rc;
    std::swap(s->fa, s->fb);
    if (!one) {
        for (int t = 1; t < nsteps - 1; ++t) {
            cudaError_t e = launch_one_step(s);
            if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
            std::swap(s->fa, s->fb);
        }
        for (int k = 0; k < S; ++k) {
            if ((rc = slab_step(s, k, S)) || (rc = slab_down(s, f_out, k, S, nd++ % R))) return rc;
        }
        std::swap(s->fa, s->fb);
    }
    s->time += nsteps;  // SimulationSetup.cpp:138
    // The handle's stream waits for the last download.
    MPH_CK(cudaStreamWaitEvent(s->stream, s->ev_slab[3 * R + (nd - 1) % R], 0), "pipeline order");
    return MPH_OK;
}

int sync(mph_sim* s, const char* what) {
    MPH_CK(cudaStreamSynchronize(s->stream), what);
    return MPH_OK;
}

}  // namespace

extern "C" {

int mph_host_alloc(long long bytes, void** out) {
    if (!out || bytes <= 0) return fail(MPH_ERR_ARG, "mph_host_alloc: bad argument");
    *out = nullptr;
    MPH_CK(cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault), "cudaHostAlloc");
    return MPH_OK;
}

int mph_host_free(void* p) {
    if (p) MPH_CK(cudaFreeHost(p), "cudaFreeHost");
    return MPH_OK;
}

int mph_set_device(int device) {
    int n = 0;
    MPH_CK(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(MPH_ERR_ARG, "mph_set_device: no such device");
    MPH_CK(cudaSetDevice(device), "cudaSetDevice");
    return MPH_OK;
}

int mph_create(const mph_desc* desc, mph_sim** out) {
    if (!desc || !out) return fail(MPH_ERR_ARG, "mph_create: NULL argument");
    *out = nullptr;
    const mph_desc& d = *desc;
    if (!lattice_ok(d.dim, d.q)) return fail(MPH_ERR_ARG, "mph_create: unsupported lattice (dim, q)");
    if (elem_size(d.precision) == 0) return fail(MPH_ERR_ARG, "mph_create: unknown precision");
    for (int a = 0; a < d.dim; ++a)
        if (d.n[a] < 1) return fail(MPH_ERR_ARG, "mph_create: cell counts must be positive");
    if (d.dim == 2 && d.n[2] != 1) return fail(MPH_ERR_ARG, "mph_create: n[2] must be 1 for a 2-D lattice");
    const long long ncell = (long long)d.n[0] * d.n[1] * (d.dim == 3 ? d.n[2] : 1);
    if (ncell >= (1LL << 31)) return fail(MPH_ERR_ARG, "mph_create: more than 2^31-1 cells");
    if ((long long)d.q * ncell >= (1LL << 32))
        return fail(MPH_ERR_ARG, "mph_create: q * cells must stay below 2^32 (32-bit element indices)");
    if ((d.dim == 3 ? d.n[2] : 1) > 65535 || d.n[1] > 65535)
        return fail(MPH_ERR_ARG, "mph_create: ny or nz exceeds the launch grid limit (65535)");
    if (!(d.omega > 0.0 && d.omega < 2.0)) return fail(MPH_ERR_CONFIG, "mph_create: omega must lie in (0, 2)");
    if (d.precision == MPH_PREC_F64X && d.forced)
        for (int a = 0; a < d.dim; ++a)
            if (!(std::fabs(d.force[a]) < 0.5 * d.omega))
                return fail(MPH_ERR_CONFIG, "mph_create: fixed-point precision needs |force| < omega / 2");
    auto* s = new mph_sim();
    s->d = d;
    if (d.dim == 2) s->d.n[2] = 1;
    int rc = resolve_table(s->d, s->table);
    if (rc) { delete s; return rc; }
    build_params(s->d, s->table, s->kp);
    s->elem = elem_size(d.precision);
    const size_t bytes = s->elem * (size_t)d.q * (size_t)ncell;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&s->fa, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->fb, bytes);
    if (e == cudaSuccess && d.precision == MPH_PREC_F16W) {  // saturation flag of the stores
        e = cudaMalloc(&s->d_flag, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(s->d_flag, 0, sizeof(int));
        s->kp.flag = s->d_flag;
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->d_kp, sizeof(KParams));
    if (e == cudaSuccess) e = cudaMemcpy(s->d_kp, &s->kp, sizeof(KParams), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && d.precision == MPH_PREC_F64X) {
        long long kbb[27 * 27];
        build_fixed_public(s->d, s->table, s->kp, s->kpx, kbb);
        e = cudaMalloc(&s->d_kbb, sizeof(kbb));
        if (e == cudaSuccess) e = cudaMemcpy(s->d_kbb, kbb, sizeof(kbb), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&s->d_flag, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(s->d_flag, 0, sizeof(int));
        // Kernel choice: one cell per thread (measured faster on GB300: 18.3
        // vs 16.5 GLUPS at 512^3 D3Q19), or the persistent cp.async pipeline
        // with MPH_F64X_KERNEL=pipe.
        const char* kv = std::getenv("MPH_F64X_KERNEL");
        if (e == cudaSuccess && kv && std::strcmp(kv, "pipe") == 0) {
            s->pipe_ctas = f64x_pipe_ctas(d.q, d.forced != 0);
            if (s->pipe_ctas <= 0) {
                e = cudaGetLastError();
                if (e == cudaSuccess) e = cudaErrorInvalidConfiguration;
            }
        }
    }
    // 16-bit storages: the pair step with bulk-copy staging of its pull
    // operands (MPH_PAIR_KERNEL=bulk, stages MPH_BULK_STAGES 2 or 3, chunk
    // cells MPH_BULK_CELLS) or the direct pair kernel (MPH_PAIR_KERNEL=direct).
    const bool p16 = d.precision == MPH_PREC_F16S || d.precision == MPH_PREC_BF16S || d.precision == MPH_PREC_F16C;
    if (e == cudaSuccess && p16) {
        const char* kv = std::getenv("MPH_PAIR_KERNEL");
        if (kv && std::strcmp(kv, "bulk") == 0) {
            s->bulk_stages = 3;
            if (const char* v = std::getenv("MPH_BULK_STAGES")) s->bulk_stages = std::atoi(v);
            if (const char* v = std::getenv("MPH_BULK_CELLS")) s->bulk_cells = std::atoi(v);
            if (s->bulk_stages < 2 || s->bulk_stages > 3 || s->bulk_cells < 2) {
                free_all(s);
                delete s;
                return fail(MPH_ERR_ARG, "mph_create: MPH_BULK_STAGES must be 2 or 3 and MPH_BULK_CELLS >= 2");
            }
            e = cudaMalloc(&s->d_flag, sizeof(int));
            if (e == cudaSuccess) e = cudaMemset(s->d_flag, 0, sizeof(int));
            if (e == cudaSuccess) e = launch_bulk(s, 0, s->kp);
        }
    }
    // Domains of up to 2^22 cells (a step of at most a few tens of
    // microseconds, where the launch cost matters) advance in runs of 32
    // steps replayed from CUDA graphs; MPH_GRAPH_STEPS sets the run length
    // (even; 0 = plain launches).
    s->graph_steps = ncell <= (1LL << 22) ? 32 : 0;
    if (const char* env = std::getenv("MPH_GRAPH_STEPS")) {
        const int g = std::atoi(env);
        s->graph_steps = (g > 0 && g % 2 == 0) ? g : 0;
    }
    s->red_blocks = 152 * 4;
    if (e == cudaSuccess) e = cudaMalloc(&s->d_part, sizeof(double) * 4 * s->red_blocks);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_red, sizeof(double) * 4);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "mph_create");
        free_all(s);
        delete s;
        return rc;
    }
    *out = s;
    return MPH_OK;
}

int mph_destroy(mph_sim* s) {
    if (!s) return MPH_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
    return MPH_OK;
}

namespace {
// A new state clears the status flag (range, saturation, wait timeout) that
// the steps of the previous state raised.
int clear_status(mph_sim* s) {
    if (s->d_flag) MPH_CK(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream), "clear status flag");
    return MPH_OK;
}
}  // namespace

int mph_set_f(mph_sim* s, const double* f) {
    if (!s || !f) return fail(MPH_ERR_ARG, "mph_set_f: NULL argument");
    int rc = clear_status(s);
    if (rc) return rc;
    rc = upload(s, f);
    if (rc) return rc;
    s->has_state = true;
    s->has_uprev = false;
    rc = sync(s, "mph_set_f");
    // a weight-scaled 16-bit store that saturated is reported here (and by
    // the steps, until a new state replaces this one)
    if (!rc && s->d.precision == MPH_PREC_F16W) rc = check_flag(s);
    return rc;
}

int mph_get_f(mph_sim* s, double* f) {
    if (!s || !f) return fail(MPH_ERR_ARG, "mph_get_f: NULL argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_get_f: no populations yet (call mph_set_f or mph_init_fields)");
    int rc = download(s, f);
    if (rc) return rc;
    return sync(s, "mph_get_f");
}

int mph_init_fields(mph_sim* s, double* rho, double* u) {
    if (!s || !rho || !u) return fail(MPH_ERR_ARG, "mph_init_fields: NULL argument");
    int rc = ensure_macro(s);
    if (!rc) rc = clear_status(s);
    if (rc) return rc;
    const long long N = s->kp.ncell;
    MPH_CK(cudaMemcpyAsync(s->d_rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream), "init upload rho");
    MPH_CK(cudaMemcpyAsync(s->d_u, u, sizeof(double) * s->d.dim * N, cudaMemcpyHostToDevice, s->stream), "init upload u");
    MPH_CK(launch_init(s->d.precision, s->d.q, s->d.forced != 0, s->fa, s->d_rho, s->d_u, s->kp, s->stream), "init kernel");
    if (s->d.forced) {
        MPH_CK(cudaMemcpyAsync(rho, s->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream), "init download rho");
        MPH_CK(cudaMemcpyAsync(u, s->d_u, sizeof(double) * s->d.dim * N, cudaMemcpyDeviceToHost, s->stream), "init download u");
    }
    s->has_state = true;
    s->has_uprev = false;
    s->time = 0.0;
    rc = sync(s, "mph_init_fields");
    if (!rc && s->d.precision == MPH_PREC_F16W) rc = check_flag(s);
    return rc;
}

int mph_init_fields_neq(mph_sim* s, const double* rho, const double* u) {
    if (!s || !rho || !u) return fail(MPH_ERR_ARG, "mph_init_fields_neq: NULL argument");
    if (s->d.forced) return fail(MPH_ERR_UNSUPPORTED, "mph_init_fields_neq: forced domains are not supported");
    int rc = ensure_macro(s);
    if (!rc) rc = clear_status(s);
    if (rc) return rc;
    const long long N = s->kp.ncell;
    MPH_CK(cudaMemcpyAsync(s->d_rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream), "init upload rho");
    MPH_CK(cudaMemcpyAsync(s->d_u, u, sizeof(double) * s->d.dim * N, cudaMemcpyHostToDevice, s->stream), "init upload u");
    MPH_CK(launch_init_neq(s->d.precision, s->d.q, s->fa, s->d_rho, s->d_u, s->kp, s->stream), "init kernel");
    s->has_state = true;
    s->has_uprev = false;
    s->time = 0.0;
    rc = sync(s, "mph_init_fields_neq");
    if (!rc && s->d.precision == MPH_PREC_F16W) rc = check_flag(s);
    return rc;
}

int mph_advance(mph_sim* s, int nsteps) {
    if (!s || nsteps < 0) return fail(MPH_ERR_ARG, "mph_advance: bad argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_advance: no populations yet");
    int rc = advance_async(s, nsteps);
    if (rc) return rc;
    rc = sync(s, "mph_advance");
    if (rc) return rc;
    return check_flag(s);
}

int mph_advance_timed(mph_sim* s, int nsteps, float* ms) {
    if (!s || nsteps < 0 || !ms) return fail(MPH_ERR_ARG, "mph_advance_timed: bad argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_advance_timed: no populations yet");
    MPH_CK(cudaEventRecord(s->ev0, s->stream), "event record");
    int rc = advance_async(s, nsteps);
    if (rc) return rc;
    MPH_CK(cudaEventRecord(s->ev1, s->stream), "event record");
    MPH_CK(cudaEventSynchronize(s->ev1), "event sync");
    MPH_CK(cudaEventElapsedTime(ms, s->ev0, s->ev1), "event elapsed");
    return check_flag(s);
}

int mph_update_macroscopic(mph_sim* s, double* rho, double* u) {
    if (!s || !rho || !u) return fail(MPH_ERR_ARG, "mph_update_macroscopic: NULL argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_update_macroscopic: no populations yet");
    int rc = ensure_macro(s);
    if (rc) return rc;
    const long long N = s->kp.ncell;
    MPH_CK(launch_moments(s->d.precision, s->d.q, s->d.forced != 0, s->fa, s->d_rho, s->d_u, s->kp, s->d_kp, s->stream),
           "moments kernel");
    MPH_CK(cudaMemcpyAsync(rho, s->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream), "download rho");
    MPH_CK(cudaMemcpyAsync(u, s->d_u, sizeof(double) * s->d.dim * N, cudaMemcpyDeviceToHost, s->stream), "download u");
    return sync(s, "mph_update_macroscopic");
}

int mph_reduce(mph_sim* s, double* out) {
    if (!s || !out) return fail(MPH_ERR_ARG, "mph_reduce: NULL argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_reduce: no populations yet");
    MPH_CK(launch_reduce(s->d.precision, s->d.q, s->fa, s->kp.ncell, s->d_part, s->red_blocks, s->d_red, s->stream),
           "reduce kernel");
    MPH_CK(cudaMemcpyAsync(out, s->d_red, sizeof(double) * 4, cudaMemcpyDeviceToHost, s->stream), "download sums");
    return sync(s, "mph_reduce");
}

int mph_set_obstacles(mph_sim* s, const unsigned char* mask) {
    if (!s) return fail(MPH_ERR_ARG, "mph_set_obstacles: NULL handle");
    if (s->pipe_ctas > 0)
        return fail(MPH_ERR_UNSUPPORTED, "mph_set_obstacles: the pipelined fixed-point kernel has no obstacle path");
    MPH_CK(cudaStreamSynchronize(s->stream), "mph_set_obstacles");
    if (!mask) {
        s->kp.cls = nullptr;
    } else {
        std::vector<unsigned char> cls(s->kp.ncell);
        build_cls(s->kp, s->d.q, mask, cls.data());
        if (!s->d_cls) MPH_CK(cudaMalloc(&s->d_cls, s->kp.ncell), "cudaMalloc(obstacle classes)");
        MPH_CK(cudaMemcpy(s->d_cls, cls.data(), s->kp.ncell, cudaMemcpyHostToDevice), "upload obstacle classes");
        s->kp.cls = s->d_cls;
    }
    MPH_CK(cudaMemcpy(s->d_kp, &s->kp, sizeof(KParams), cudaMemcpyHostToDevice), "upload parameters");
    drop_graphs(s);  // the captured launches carry the old parameters
    return MPH_OK;
}

int mph_residual(mph_sim* s, double* out) {
    if (!s || !out) return fail(MPH_ERR_ARG, "mph_residual: NULL argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_residual: no populations yet");
    if (!s->d_uprev)
        MPH_CK(cudaMalloc(&s->d_uprev, sizeof(double) * s->d.dim * s->kp.ncell), "cudaMalloc(residual field)");
    MPH_CK(launch_residual(s->d.precision, s->d.q, s->fa, s->kp.ncell, s->d_uprev, !s->has_uprev, s->d_part,
                           s->red_blocks, s->d_red, s->stream),
           "residual kernel");
    double sums[2];
    MPH_CK(cudaMemcpyAsync(sums, s->d_red, sizeof(sums), cudaMemcpyDeviceToHost, s->stream), "download residual");
    int rc = sync(s, "mph_residual");
    if (rc) return rc;
    out[1] = std::sqrt(sums[1]);
    out[0] = relative_change(sums[0], sums[1], s->has_uprev);
    s->has_uprev = true;
    return MPH_OK;
}

int mph_lattice(int q, int* c, double* w, int* opp) {
    switch (q) {
        case 9: lattice_tables<9>(c, w, opp); return MPH_OK;
        case 15: lattice_tables<15>(c, w, opp); return MPH_OK;
        case 19: lattice_tables<19>(c, w, opp); return MPH_OK;
        case 27: lattice_tables<27>(c, w, opp); return MPH_OK;
    }
    return fail(MPH_ERR_ARG, "mph_lattice: q must be 9, 15, 19 or 27");
}

int mph_state_bytes(const mph_sim* s, long long* bytes) {
    if (!s || !bytes) return fail(MPH_ERR_ARG, "mph_state_bytes: NULL argument");
    *bytes = (long long)(s->elem * (size_t)s->d.q * (size_t)s->kp.ncell);
    return MPH_OK;
}

int mph_get_state(mph_sim* s, void* buf, long long bytes) {
    if (!s || !buf) return fail(MPH_ERR_ARG, "mph_get_state: NULL argument");
    if (!s->has_state) return fail(MPH_ERR_STATE, "mph_get_state: no populations yet");
    const long long n = (long long)(s->elem * (size_t)s->d.q * (size_t)s->kp.ncell);
    if (bytes != n) return fail(MPH_ERR_ARG, "mph_get_state: size differs from mph_state_bytes");
    MPH_CK(cudaMemcpyAsync(buf, s->fa, (size_t)n, cudaMemcpyDeviceToHost, s->stream), "download state");
    return sync(s, "mph_get_state");
}

int mph_set_state(mph_sim* s, const void* buf, long long bytes) {
    if (!s || !buf) return fail(MPH_ERR_ARG, "mph_set_state: NULL argument");
    const long long n = (long long)(s->elem * (size_t)s->d.q * (size_t)s->kp.ncell);
    if (bytes != n) return fail(MPH_ERR_ARG, "mph_set_state: size differs from mph_state_bytes");
    const int rc = clear_status(s);
    if (rc) return rc;
    MPH_CK(cudaMemcpyAsync(s->fa, buf, (size_t)n, cudaMemcpyHostToDevice, s->stream), "upload state");
    s->has_state = true;
    s->has_uprev = false;
    return sync(s, "mph_set_state");
}

int mph_set_time(mph_sim* s, double t) {
    if (!s) return fail(MPH_ERR_ARG, "mph_set_time: NULL handle");
    s->time = t;
    return MPH_OK;
}

int mph_time(const mph_sim* s, double* t) {
    if (!s || !t) return fail(MPH_ERR_ARG, "mph_time: NULL argument");
    *t = s->time;
    return MPH_OK;
}

int mph_launches_per_step(const mph_sim* s, int* n) {
    if (!s || !n) return fail(MPH_ERR_ARG, "mph_launches_per_step: NULL argument");
    *n = 1;
    return MPH_OK;
}

int mph_step_host(mph_sim* s, const double* f_in, double* f_out, int nsteps) {
    if (!s || !f_in || !f_out || nsteps < 0) return fail(MPH_ERR_ARG, "mph_step_host: bad argument");
    s->has_uprev = false;  // the state is replaced, as by mph_set_f
    const int S = nsteps > 0 ? slab_count(s) : 0;
    if (S > 0) {
        s->has_state = true;
        int rc = step_host_slabs(s, f_in, f_out, nsteps, S);
        if (rc) {
            // Copies already queued may still touch the caller's buffers:
            // let them finish before the error reaches the caller.
            for (cudaStream_t st : {s->copy_stream, s->conv_stream, s->d2h_stream, s->stream})
                if (st) cudaStreamSynchronize(st);
            return rc;
        }
        rc = sync(s, "mph_step_host");
        return rc ? rc : check_flag(s);
    }
    int rc = upload(s, f_in);
    if (rc) return rc;
    s->has_state = true;
    rc = advance_async(s, nsteps);
    if (rc) return rc;
    rc = download(s, f_out);
    if (rc) return rc;
    rc = sync(s, "mph_step_host");
    if (rc) return rc;
    return check_flag(s);
}

// ---- plugin level ------------------------------------------------------
static int to_a4(const mph_array4* a, A4& o, int q, const char* what) {
    if (!a || !a->p) return fail(MPH_ERR_ARG, std::string(what) + ": NULL Array4");
    if (a->ncomp < q) return fail(MPH_ERR_ARG, std::string(what) + ": Array4 has fewer than Q components");
    o.p = a->p;
    o.js = a->jstride; o.ks = a->kstride; o.ns = a->nstride;
    for (int d = 0; d < 3; ++d) {
        o.b[d] = a->begin[d];
        o.e[d] = a->end[d];
        if (o.e[d] <= o.b[d]) return fail(MPH_ERR_ARG, std::string(what) + ": empty Array4 extent");
    }
    return MPH_OK;
}

static bool a4_contains(const A4& a, const int lo[3], const int hi[3]) {
    for (int d = 0; d < 3; ++d)
        if (lo[d] < a.b[d] || hi[d] >= a.e[d]) return false;
    return true;
}

int mph_pull_collide_fused_arr(int dim, int q, const int lo[3], const int hi[3], const mph_array4* fin,
                               const mph_array4* fout, double omega, const double* force, void* stream) {
    if (!lattice_ok(dim, q) || !lo || !hi) return fail(MPH_ERR_ARG, "mph_pull_collide_fused_arr: bad lattice or box");
    A4 a, b;
    int rc = to_a4(fin, a, q, "mph_pull_collide_fused_arr(fin)");
    if (rc) return rc;
    rc = to_a4(fout, b, q, "mph_pull_collide_fused_arr(fout)");
    if (rc) return rc;
    int l[3] = {lo[0], lo[1], dim == 3 ? lo[2] : 0}, h[3] = {hi[0], hi[1], dim == 3 ? hi[2] : 0};
    for (int d = 0; d < dim; ++d)
        if (h[d] < l[d]) return fail(MPH_ERR_ARG, "mph_pull_collide_fused_arr: empty box");
    int gl[3] = {l[0] - 1, l[1] - 1, dim == 3 ? l[2] - 1 : l[2]}, gh[3] = {h[0] + 1, h[1] + 1, dim == 3 ? h[2] + 1 : h[2]};
    if (!a4_contains(a, gl, gh)) return fail(MPH_ERR_ARG, "mph_pull_collide_fused_arr: fin does not cover box grown by 1");
    if (!a4_contains(b, l, h)) return fail(MPH_ERR_ARG, "mph_pull_collide_fused_arr: fout does not cover the box");
    mph_desc d;
    std::memset(&d, 0, sizeof(d));
    d.dim = dim; d.q = q; d.omega = omega; d.forced = force != nullptr;
    d.n[0] = h[0] - l[0] + 1; d.n[1] = h[1] - l[1] + 1; d.n[2] = h[2] - l[2] + 1;
    for (int a2 = 0; a2 < 3; ++a2) d.force[a2] = (force && a2 < dim) ? force[a2] : 0.0;
    for (int f = 0; f < 6; ++f) d.face_type[f] = MPH_BC_PERIODIC;
    mph_resolved_bc tab[27];
    for (int c = 0; c < 27; ++c) { tab[c].type = MPH_BC_PERIODIC; tab[c].rho = 1.0; tab[c].U[0] = tab[c].U[1] = tab[c].U[2] = 0.0; }
    KParams kp;
    build_params(d, tab, kp);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPH_CK(launch_pull_collide_arr(dim, q, force != nullptr, l, h, a, b, kp, st), "pull_collide_arr");
    MPH_CK(cudaStreamSynchronize(st), "pull_collide_arr sync");
    return MPH_OK;
}

int mph_periodic_fill_arr(int dim, int q, const int dom_lo[3], const int dom_hi[3], const int periodic[3],
                          const mph_array4* f, void* stream) {
    if (!lattice_ok(dim, q) || !dom_lo || !dom_hi || !periodic) return fail(MPH_ERR_ARG, "mph_periodic_fill_arr: bad argument");
    A4 a;
    int rc = to_a4(f, a, q, "mph_periodic_fill_arr");
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPH_CK(launch_periodic_fill_arr(dim, q, dom_lo, dom_hi, periodic, a, st), "periodic_fill_arr");
    MPH_CK(cudaStreamSynchronize(st), "periodic_fill_arr sync");
    return MPH_OK;
}

int mph_bc_fill_arr(int dim, int q, const int dom_lo[3], const int dom_hi[3], const int periodic[3],
                    const mph_resolved_bc* table, const mph_array4* f, void* stream) {
    if (!lattice_ok(dim, q) || !dom_lo || !dom_hi || !periodic || !table)
        return fail(MPH_ERR_ARG, "mph_bc_fill_arr: bad argument");
    A4 a;
    int rc = to_a4(f, a, q, "mph_bc_fill_arr");
    if (rc) return rc;
    KParams kp;
    std::memset(&kp, 0, sizeof(kp));
    for (int c = 0; c < 27; ++c) {
        if (table[c].type < 0 || table[c].type > MPH_BC_PERIODIC) return fail(MPH_ERR_ARG, "mph_bc_fill_arr: bad table type");
        kp.bc_type[c] = table[c].type;
        kp.bc_rho[c] = table[c].rho;
        for (int k = 0; k < 3; ++k) kp.bc_U[c][k] = table[c].U[k];
    }
    KParams* dkp = nullptr;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPH_CK(cudaMalloc(&dkp, sizeof(KParams)), "bc_fill_arr params");
    cudaError_t e = cudaMemcpyAsync(dkp, &kp, sizeof(KParams), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_bc_fill_arr(dim, q, dom_lo, dom_hi, periodic, dkp, a, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dkp);
    if (e != cudaSuccess) return cuda_fail(e, "bc_fill_arr");
    return MPH_OK;
}

}  // extern "C"
