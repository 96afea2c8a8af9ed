// batch.cu -- many independent domains of uneven sizes advanced together.
//
// The reference advances one domain per process; a parameter sweep or an
// ensemble (hundreds of lid-driven cavities of different size and Reynolds
// number) would run hundreds of solver instances.  Here all domains share one
// population buffer (domain-major, then population, then cell) and one kernel
// per step covers every domain: the grid is a flat list of chunks of 256 K
// consecutive cells, each naming its domain, so the work is balanced across
// the 152 SMs however uneven the domains are, and no lane idles on a ragged
// domain edge.  Each domain's constants (KParams: size, omega,
// boundary table) sit in global memory and are read by the same pull /
// collide device code as a single domain, so every domain's result is
// bit-identical to a single-domain handle with the same description.
//
// Step pairs are captured once as CUDA graphs and replayed: one graph per
// buffer the state starts in (A->B->A and B->A->B), chosen at each replay,
// so an odd number of steps before a replay keeps the right input.
// K (cells per thread) is chosen by an autotuner that times the candidates
// on the batch itself and caches the winner per (Q, precision, size class).
// mph_batch_advance_looped_timed runs the same steps as one launch per domain
// per step, the baseline the batched kernel is compared with.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "batch_kernel.cuh"
#include "lbm_launch.h"
#include "mph_internal.h"

using namespace mph;

namespace {

// dpx, kbb and flag are used by the fixed-point precision only.
cudaError_t launch_batch(int prec, int q, bool forced, int K, bool P, const void* fin, void* fout, const Chunk* chunks,
                         int nchunks, const int2* walls, int nwalls, const KParams* dp, const long long* offs,
                         const KParamsX* dpx, const long long* kbb, int* flag, cudaStream_t s) {
    switch (prec) {
        case MPH_PREC_F64X:
            return launch_batch_f64x(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, dpx, offs, kbb,
                                     flag, s);
        case MPH_PREC_F64:
            return launch_batch_exact(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_F64_FAST:
            return launch_batch_fast_f64(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_F32: return launch_batch_f32(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_F16S: return launch_batch_f16s(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_BF16S:
            return launch_batch_bf16s(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_F16C:
            return launch_batch_f16c(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
        case MPH_PREC_F16W:
            return launch_batch_f16w(q, forced, K, P, fin, fout, chunks, nchunks, walls, nwalls, dp, offs, s);
    }
    return cudaErrorInvalidValue;
}

size_t elem_of(int prec) {
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

// Candidates of the autotuner: cand % 3 selects K, the cells per thread (a
// chunk is 256 K cells), cand / 3 a persistent grid; the shifted 16-bit
// policies take cells in pairs, so K = 1 is skipped for them, and the
// fixed-point step holds at most two cells of int64 populations per thread,
// so K = 4 is skipped for it.  Candidate 6 (16-bit storages only, chosen
// only through MPH_BATCH_CANDIDATE=6) is the persistent kernel with
// bulk-copy staging over chunks of whole rows: bit-identical, but measured
// slower than the direct kernels (the 16-bit step is bound by instruction
// issue, and staging adds instructions), so the autotuner does not time it.
constexpr int kCells[3] = {1, 2, 4};
constexpr int kCands = 7;
constexpr int kBulkCand = 6;
constexpr int kBulkCells = 512;  // cells per row chunk of the staged kernel
constexpr int kBulkStages = 3;

bool shifted(int prec) {
    return prec == MPH_PREC_F16S || prec == MPH_PREC_BF16S || prec == MPH_PREC_F16C || prec == MPH_PREC_F16W;
}
// Per-domain status flags: the fixed-point range flag and the saturation
// flag of the weight-scaled 16-bit storage.
bool per_domain_flags(int prec) { return prec == MPH_PREC_F64X || prec == MPH_PREC_F16W; }
bool candidate_ok(int prec, int cand) {
    if (cand == kBulkCand) return shifted(prec) && prec != MPH_PREC_F16W;
    if (shifted(prec)) return cand % 3 != 0;
    if (prec == MPH_PREC_F64X) return cand % 3 != 2;
    return true;
}

// Autotuner cache: (q, precision, log2 total cells, log2 domains) -> K index.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tune;

}  // namespace

// Defined in sim.cu (shared with single domains).
namespace mph {
void build_params_public(const mph_desc& d, const mph_resolved_bc* tab, KParams& kp);
void build_fixed_public(const mph_desc& d, const mph_resolved_bc* tab, const KParams& kp, KParamsX& px,
                        long long* kbb);
void build_cls(const KParams& p, int q, const unsigned char* mask, unsigned char* cls);
}
namespace mph {
double relative_change(double s0, double s1, bool has_prev);
}

struct mph_batch {
    int ndom = 0, q = 0, dim = 0, prec = 0;
    bool forced = false;
    std::vector<mph_desc> descs;
    std::vector<long long> offs_h;  // element offset of each domain
    long long total_elems = 0, total_cells = 0;
    KParams* d_params = nullptr;
    long long* d_offs = nullptr;
    void* fa = nullptr;
    void* fb = nullptr;
    double* d_stage = nullptr;
    double* d_rho = nullptr;
    double* d_u = nullptr;
    long long max_cells = 0;
    std::vector<KParams> params_h;
    // fixed-point precision: per-domain constants, bounce-back tables
    // (27 x 27 per domain) and the range flags of the step kernels (one per
    // domain on the device, cleared after each read; bad_h keeps them on the
    // host until the domain is initialised or its populations replaced)
    std::vector<KParamsX> px_h;
    KParamsX* d_px = nullptr;
    long long* d_kbb = nullptr;
    int* d_flag = nullptr;
    std::vector<int> bad_h;
    // cells needing the boundary rules {domain, cell}
    int2* d_walls = nullptr;
    int nwalls = 0;
    // obstacle classes per domain (host copies; empty = none) and on the device
    std::vector<std::vector<unsigned char>> cls_h;
    unsigned char* d_cls = nullptr;
    std::vector<long long> coffs_h;  // cell offset of each domain
    // chunk lists per candidate K, and the index of each domain's first chunk
    Chunk* d_chunks[3] = {nullptr, nullptr, nullptr};
    int nchunks[3] = {0, 0, 0};
    int* d_chunk_first[3] = {nullptr, nullptr, nullptr};
    // steady-state residual: saved velocity (dim x cells, domain-major), cell
    // offsets, partials per chunk and per-domain sums
    double* d_uprev = nullptr;
    long long* d_coffs = nullptr;
    double* d_rpart = nullptr;
    double* d_rout = nullptr;
    bool has_uprev = false;
    int k_idx = -1;  // candidate chosen by the autotuner
    // 16-bit storages: row chunks of the bulk-copy staged kernel (candidate
    // 6), its run slot length and whether it fits in shared memory
    RowChunk* d_rchunks = nullptr;
    int nrchunks = 0, bulk_lpad = 0;
    bool bulk_ok = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // two steps from graph_in[i] back to it
    void* graph_in[2] = {nullptr, nullptr};          // the buffer graph[i] starts from
    int graph_k = -1;
    double time = 0.0;
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

void free_batch(mph_batch* b) {
    cudaFree(b->d_params);
    cudaFree(b->d_offs);
    cudaFree(b->fa);
    cudaFree(b->fb);
    cudaFree(b->d_stage);
    cudaFree(b->d_rho);
    cudaFree(b->d_u);
    for (auto* t : b->d_chunks) cudaFree(t);
    for (auto* t : b->d_chunk_first) cudaFree(t);
    cudaFree(b->d_uprev);
    cudaFree(b->d_coffs);
    cudaFree(b->d_rpart);
    cudaFree(b->d_rout);
    cudaFree(b->d_walls);
    cudaFree(b->d_cls);
    cudaFree(b->d_rchunks);
    cudaFree(b->d_px);
    cudaFree(b->d_kbb);
    cudaFree(b->d_flag);
    for (cudaGraphExec_t g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
}

int ensure_chunks(mph_batch* b, int ki) {
    if (b->d_chunks[ki]) return MPH_OK;
    const long long len = 256LL * kCells[ki];
    std::vector<Chunk> chunks;
    std::vector<int> first(b->ndom + 1, 0);
    for (int d = 0; d < b->ndom; ++d) {
        first[d] = (int)chunks.size();
        const mph_desc& ds = b->descs[d];
        const long long nx = ds.n[0], ny = ds.n[1];
        const long long cells = nx * ny * (ds.dim == 3 ? ds.n[2] : 1);
        for (long long c = 0; c < cells; c += len) {
            const long long row = c / nx;
            chunks.push_back(Chunk{d, (int)c, (int)(c - row * nx), (int)((row % ny) | ((row / ny) << 16))});
        }
    }
    if (chunks.size() > 0x7fffffffu) return fail(MPH_ERR_ARG, "batch: too many chunks");
    first[b->ndom] = (int)chunks.size();
    MPH_CK(cudaMalloc(&b->d_chunk_first[ki], sizeof(int) * first.size()), "batch chunk index");
    MPH_CK(cudaMemcpy(b->d_chunk_first[ki], first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice),
           "batch chunk index");
    MPH_CK(cudaMalloc(&b->d_chunks[ki], sizeof(Chunk) * chunks.size()), "batch chunks");
    MPH_CK(cudaMemcpy(b->d_chunks[ki], chunks.data(), sizeof(Chunk) * chunks.size(), cudaMemcpyHostToDevice),
           "batch chunks");
    b->nchunks[ki] = (int)chunks.size();
    return MPH_OK;
}

// The list of cells whose pulls need the boundary rules: cells next to a
// non-periodic face (whole rows on y / z faces, the row ends on x faces) and
// obstacle cells with their fluid neighbours.
int build_walls(mph_batch* b) {
    std::vector<int2> walls;
    for (int d = 0; d < b->ndom; ++d) {
        const KParams& p = b->params_h[d];
        const unsigned char* cls = b->cls_h[d].empty() ? nullptr : b->cls_h[d].data();
        for (int z = 0; z < p.nz; ++z)
            for (int y = 0; y < p.ny; ++y) {
                const int row = (z * p.ny + y) * p.nx;
                const bool face = (!p.periodic[1] && (y == 0 || y == p.ny - 1)) ||
                                  (b->dim == 3 && !p.periodic[2] && (z == 0 || z == p.nz - 1));
                for (int x = 0; x < p.nx; ++x) {
                    const bool edge = face || (!p.periodic[0] && (x == 0 || x == p.nx - 1)) ||
                                      (cls && cls[row + x] != kFluid);
                    if (edge) walls.push_back(make_int2(d, row + x));
                }
            }
    }
    if (walls.size() > 0x7fffffffu) return fail(MPH_ERR_ARG, "batch: too many wall cells");
    cudaFree(b->d_walls);
    b->d_walls = nullptr;
    b->nwalls = (int)walls.size();
    if (walls.empty()) return MPH_OK;
    MPH_CK(cudaMalloc(&b->d_walls, sizeof(int2) * walls.size()), "batch wall list");
    MPH_CK(cudaMemcpy(b->d_walls, walls.data(), sizeof(int2) * walls.size(), cudaMemcpyHostToDevice), "batch wall list");
    return MPH_OK;
}

cudaError_t launch_bulk(mph_batch* b, int mode) {
    switch (b->prec) {
        case MPH_PREC_F16S:
            return launch_batch_bulk_f16s(mode, b->q, b->forced, kBulkStages, b->bulk_lpad, b->fa, b->fb, b->d_rchunks,
                                          b->nrchunks, b->d_walls, b->nwalls, b->d_params, b->d_offs, b->d_flag,
                                          b->stream);
        case MPH_PREC_BF16S:
            return launch_batch_bulk_bf16s(mode, b->q, b->forced, kBulkStages, b->bulk_lpad, b->fa, b->fb, b->d_rchunks,
                                           b->nrchunks, b->d_walls, b->nwalls, b->d_params, b->d_offs, b->d_flag,
                                           b->stream);
        case MPH_PREC_F16C:
            return launch_batch_bulk_f16c(mode, b->q, b->forced, kBulkStages, b->bulk_lpad, b->fa, b->fb, b->d_rchunks,
                                          b->nrchunks, b->d_walls, b->nwalls, b->d_params, b->d_offs, b->d_flag,
                                          b->stream);
    }
    return cudaErrorNotSupported;
}

// Row chunks of the staged kernel (about kBulkCells cells of whole rows per
// chunk), the longest run slot, and the kernel's shared-memory setting.
int build_row_chunks(mph_batch* b) {
    std::vector<RowChunk> rc;
    long long lpad = 0;
    for (int d = 0; d < b->ndom; ++d) {
        const mph_desc& ds = b->descs[d];
        const int nx = ds.n[0], ny = ds.n[1], nz = ds.dim == 3 ? ds.n[2] : 1;
        int rows = kBulkCells / nx;
        if (rows < 1) rows = 1;
        if (rows > ny) rows = ny;
        lpad = std::max(lpad, ((long long)rows * nx + 14 + 7) & ~7LL);
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; y += rows) rc.push_back(RowChunk{d, z, y, std::min(rows, ny - y)});
    }
    if (rc.size() > 0x7fffffffu || lpad > (1 << 20)) return MPH_OK;  // the staged kernel does not apply
    b->bulk_lpad = (int)lpad;
    MPH_CK(cudaMalloc(&b->d_rchunks, sizeof(RowChunk) * rc.size()), "batch row chunks");
    MPH_CK(cudaMemcpy(b->d_rchunks, rc.data(), sizeof(RowChunk) * rc.size(), cudaMemcpyHostToDevice), "batch row chunks");
    b->nrchunks = (int)rc.size();
    if (!b->d_flag) {
        MPH_CK(cudaMalloc(&b->d_flag, sizeof(int)), "batch flag");
        MPH_CK(cudaMemset(b->d_flag, 0, sizeof(int)), "batch flag");
    }
    const cudaError_t e = launch_bulk(b, 0);
    if (e == cudaErrorNotSupported) return MPH_OK;  // runs too long for shared memory
    MPH_CK(e, "batch staged kernel setup");
    b->bulk_ok = true;
    return MPH_OK;
}

int step_once(mph_batch* b, int cand) {
    if (cand == kBulkCand) {
        MPH_CK(launch_bulk(b, 1), "batch staged step launch");
        std::swap(b->fa, b->fb);
        return MPH_OK;
    }
    const int ki = cand % 3;
    MPH_CK(launch_batch(b->prec, b->q, b->forced, kCells[ki], cand >= 3, b->fa, b->fb, b->d_chunks[ki], b->nchunks[ki],
                        b->d_walls, b->nwalls, b->d_params, b->d_offs, b->d_px, b->d_kbb, b->d_flag, b->stream),
           "batch step launch");
    std::swap(b->fa, b->fb);
    return MPH_OK;
}

// Times each candidate K on the batch itself (4 steps after 2) and keeps the
// fastest; the choice is cached per (q, precision, size class, domain-count
// class).  An even number of steps is run per candidate so the state ends in
// buffer A, and the state is restored afterwards.
int autotune(mph_batch* b) {
    if (b->k_idx >= 0) return MPH_OK;
    // MPH_BATCH_CANDIDATE=c (0..5) fixes the launch instead of timing.
    if (const char* env = std::getenv("MPH_BATCH_CANDIDATE")) {
        const int c = std::atoi(env);
        if (c < 0 || c >= kCands || !candidate_ok(b->prec, c) || (c == kBulkCand && !b->bulk_ok))
            return fail(MPH_ERR_ARG, "MPH_BATCH_CANDIDATE must be 0..6 (1, 2, 4, 5 and 6 for 16-bit storage; "
                                     "0, 1, 3, 4 for fixed point; 0..5 otherwise)");
        b->k_idx = c;
        return ensure_chunks(b, c % 3);
    }
    const int cls = (int)std::floor(std::log2((double)b->total_cells));
    const int dcls = (int)std::floor(std::log2((double)b->ndom));
    const auto key = std::make_tuple(b->q, b->prec, cls, dcls);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) b->k_idx = it->second;
    }
    if (b->k_idx >= 0) return ensure_chunks(b, b->k_idx % 3);
    // Snapshot the state so tuning does not advance the simulation.
    void* save = nullptr;
    const size_t bytes = elem_of(b->prec) * (size_t)b->total_elems;
    MPH_CK(cudaMalloc(&save, bytes), "autotune snapshot");
    cudaError_t e = cudaMemcpyAsync(save, b->fa, bytes, cudaMemcpyDeviceToDevice, b->stream);
    float best = 1e30f;
    int besti = shifted(b->prec) ? 1 : 0;
    for (int wi = 0; wi < kCands && e == cudaSuccess; ++wi) {
        if (!candidate_ok(b->prec, wi) || wi == kBulkCand) continue;
        int rc = ensure_chunks(b, wi % 3);
        if (rc) { cudaFree(save); return rc; }
        rc = step_once(b, wi);
        if (!rc) rc = step_once(b, wi);
        if (rc) { cudaFree(save); return rc; }
        e = cudaEventRecord(b->ev0, b->stream);
        for (int k = 0; k < 4 && !rc; ++k) rc = step_once(b, wi);
        if (rc) { cudaFree(save); return rc; }
        if (e == cudaSuccess) e = cudaEventRecord(b->ev1, b->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        if (e == cudaSuccess && ms < best) { best = ms; besti = wi; }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->fa, save, bytes, cudaMemcpyDeviceToDevice, b->stream);
    // only the steps of the caller's advances report the range flag
    if (e == cudaSuccess && b->d_flag)
        e = cudaMemsetAsync(b->d_flag, 0, sizeof(int) * (per_domain_flags(b->prec) ? b->ndom : 1), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(save);
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    b->k_idx = besti;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = besti;
    return MPH_OK;
}

void drop_graphs(mph_batch* b) {
    for (int i = 0; i < 2; ++i) {
        if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
        b->graph[i] = nullptr;
        b->graph_in[i] = nullptr;
    }
    b->graph_k = -1;
}

// Two steps captured as a CUDA graph for each buffer the state can start in
// (A->B->A and B->A->B).  Capture only records the launches; the two host-side
// swaps of step_once cancel, and fa / fb are put back as they were.
int ensure_graph(mph_batch* b) {
    if (b->graph[0] && b->graph[1] && b->graph_k == b->k_idx) return MPH_OK;
    drop_graphs(b);
    void* const fa0 = b->fa;
    void* const fb0 = b->fb;
    for (int i = 0; i < 2; ++i) {
        b->fa = i == 0 ? fa0 : fb0;
        b->fb = i == 0 ? fb0 : fa0;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? MPH_OK : cuda_fail(e, "graph capture begin");
        if (!rc) {
            rc = step_once(b, b->k_idx);
            if (!rc) rc = step_once(b, b->k_idx);
            e = cudaStreamEndCapture(b->stream, &g);
            if (!rc && e != cudaSuccess) rc = cuda_fail(e, "graph capture end");
        }
        if (!rc) {
            e = cudaGraphInstantiate(&b->graph[i], g, 0);
            if (e != cudaSuccess) rc = cuda_fail(e, "graph instantiate");
        }
        if (g) cudaGraphDestroy(g);
        b->graph_in[i] = i == 0 ? fa0 : fb0;
        b->fa = fa0;
        b->fb = fb0;
        if (rc) {
            drop_graphs(b);
            return rc;
        }
    }
    b->graph_k = b->k_idx;
    return MPH_OK;
}

// Range flags of the fixed-point step and saturation flags of the
// weight-scaled 16-bit storage, one per domain (read and cleared after an
// advance, kept in bad_h).
int check_flag(mph_batch* b) {
    if (!b->d_flag) return MPH_OK;
    if (!per_domain_flags(b->prec)) {  // the staged 16-bit kernel: 2 = a wait timed out
        int f = 0;
        MPH_CK(cudaMemcpyAsync(&f, b->d_flag, sizeof(int), cudaMemcpyDeviceToHost, b->stream), "read flag");
        MPH_CK(cudaStreamSynchronize(b->stream), "read flag");
        if (!f) return MPH_OK;
        MPH_CK(cudaMemsetAsync(b->d_flag, 0, sizeof(int), b->stream), "clear flag");
        return fail(MPH_ERR_CUDA, "staged 16-bit batch step: a wait for bulk-copied operands exceeded its time limit "
                                  "(the step's results are incomplete)");
    }
    std::vector<int> flag(b->ndom, 0);
    MPH_CK(cudaMemcpyAsync(flag.data(), b->d_flag, sizeof(int) * b->ndom, cudaMemcpyDeviceToHost, b->stream),
           "read flag");
    MPH_CK(cudaStreamSynchronize(b->stream), "read flag");
    int nbad = 0, first = -1;
    for (int d = 0; d < b->ndom; ++d)
        if (flag[d]) {
            b->bad_h[d] = 1;
            ++nbad;
            if (first < 0) first = d;
        }
    if (nbad) {
        MPH_CK(cudaMemsetAsync(b->d_flag, 0, sizeof(int) * b->ndom, b->stream), "clear flag");
        if (b->prec == MPH_PREC_F16W)
            return fail(MPH_ERR_NONFINITE, "weight-scaled 16-bit batch step: a population of " + std::to_string(nbad) +
                                               " domain(s) (first: " + std::to_string(first) +
                                               ") saturated (|f - w| reached the format's range, or was not "
                                               "finite); mph_batch_range_flags lists them");
        return fail(MPH_ERR_NONFINITE, "fixed-point batch step: a cell of " + std::to_string(nbad) +
                                           " domain(s) (first: " + std::to_string(first) +
                                           ") left the representable range (rho outside (1/16, 64) or |J|, "
                                           "|u| >= 4); mph_batch_range_flags lists them");
    }
    return MPH_OK;
}

int advance_batch(mph_batch* b, int nsteps) {
    int rc = autotune(b);
    if (rc) return rc;
    rc = ensure_graph(b);
    if (rc) return rc;
    // The graph that starts from the buffer holding the state now.
    const cudaGraphExec_t pair = b->fa == b->graph_in[0] ? b->graph[0] : b->graph[1];
    for (int t = 0; t + 1 < nsteps; t += 2) MPH_CK(cudaGraphLaunch(pair, b->stream), "graph launch");
    if (nsteps % 2) {
        rc = step_once(b, b->k_idx);
        if (rc) return rc;
    }
    b->time += nsteps;
    return MPH_OK;
}

}  // namespace

extern "C" {

int mph_batch_create(int ndomains, const mph_desc* descs, mph_batch** out) {
    if (ndomains < 1 || !descs || !out) return fail(MPH_ERR_ARG, "mph_batch_create: bad argument");
    *out = nullptr;
    auto* b = new mph_batch();
    b->ndom = ndomains;
    b->q = descs[0].q;
    b->dim = descs[0].dim;
    b->prec = descs[0].precision;
    b->forced = descs[0].forced != 0;
    if (elem_of(b->prec) == 0) { delete b; return fail(MPH_ERR_UNSUPPORTED, "mph_batch_create: precision not supported in a batch"); }
    b->descs.assign(descs, descs + ndomains);
    b->params_h.resize(ndomains);
    std::vector<long long> kbb_h;  // fixed-point bounce-back tables
    b->cls_h.resize(ndomains);
    long long off = 0;
    for (int d = 0; d < ndomains; ++d) {
        mph_desc& ds = b->descs[d];
        if (ds.q != b->q || ds.dim != b->dim || ds.precision != b->prec || (ds.forced != 0) != b->forced) {
            delete b;
            return fail(MPH_ERR_ARG, "mph_batch_create: all domains must share lattice, precision and forcing");
        }
        if (!lattice_ok(ds.dim, ds.q)) { delete b; return fail(MPH_ERR_ARG, "mph_batch_create: unsupported lattice"); }
        if (ds.dim == 2) ds.n[2] = 1;
        for (int a = 0; a < ds.dim; ++a)
            if (ds.n[a] < 1) { delete b; return fail(MPH_ERR_ARG, "mph_batch_create: cell counts must be positive"); }
        if (!(ds.omega > 0.0 && ds.omega < 2.0)) { delete b; return fail(MPH_ERR_CONFIG, "mph_batch_create: omega must lie in (0, 2)"); }
        if (ds.precision == MPH_PREC_F64X && ds.forced)
            for (int a = 0; a < ds.dim; ++a)
                if (!(std::fabs(ds.force[a]) < 0.5 * ds.omega)) {
                    delete b;
                    return fail(MPH_ERR_CONFIG, "mph_batch_create: fixed-point precision needs |force| < omega / 2");
                }
        // Chunk coordinates pack y | z << 16 and divide by float reciprocals;
        // element indices within a domain are 32-bit.
        if (ds.n[0] > (1 << 23) || ds.n[1] > 65535 || ds.n[2] > 32767 ||
            (long long)ds.q * ds.n[0] * ds.n[1] * ds.n[2] >= (1LL << 32)) {
            delete b;
            return fail(MPH_ERR_ARG, "mph_batch_create: domain too large for a batch (nx <= 2^23, ny <= 65535, "
                                     "nz <= 32767, q * cells < 2^32)");
        }
        mph_resolved_bc tab[27];
        int rc = resolve_table(ds, tab);
        if (rc) { delete b; return rc; }
        build_params_public(ds, tab, b->params_h[d]);
        if (b->prec == MPH_PREC_F64X) {
            b->px_h.resize(ndomains);
            kbb_h.resize((size_t)ndomains * 27 * 27);
            build_fixed_public(ds, tab, b->params_h[d], b->px_h[d], kbb_h.data() + (size_t)d * 27 * 27);
        }
        const long long cells = (long long)ds.n[0] * ds.n[1] * ds.n[2];
        b->offs_h.push_back(off);
        b->coffs_h.push_back(b->total_cells);
        // Each domain starts on a 128-element boundary (>= 256 B): aligned
        // rows for every precision and the 32-bit pair accesses of the
        // 16-bit kernels in the per-domain (looped) launches.
        off += (cells * ds.q + 127) / 128 * 128;
        b->total_cells += cells;
        b->max_cells = cells > b->max_cells ? cells : b->max_cells;
    }
    b->total_elems = off;
    const size_t bytes = elem_of(b->prec) * (size_t)off;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&b->fa, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->fb, bytes);
    if (e == cudaSuccess && b->prec == MPH_PREC_F16W) {  // per-domain saturation flags
        e = cudaMalloc(&b->d_flag, sizeof(int) * ndomains);
        if (e == cudaSuccess) e = cudaMemset(b->d_flag, 0, sizeof(int) * ndomains);
        for (int d = 0; d < ndomains; ++d) b->params_h[d].flag = b->d_flag + d;
        b->bad_h.assign(ndomains, 0);
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_params, sizeof(KParams) * ndomains);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_params, b->params_h.data(), sizeof(KParams) * ndomains, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offs, sizeof(long long) * ndomains);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_offs, b->offs_h.data(), sizeof(long long) * ndomains, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && b->prec == MPH_PREC_F64X) {
        e = cudaMalloc(&b->d_px, sizeof(KParamsX) * ndomains);
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_px, b->px_h.data(), sizeof(KParamsX) * ndomains, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_kbb, sizeof(long long) * kbb_h.size());
        if (e == cudaSuccess)
            e = cudaMemcpy(b->d_kbb, kbb_h.data(), sizeof(long long) * kbb_h.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_flag, sizeof(int) * ndomains);
        if (e == cudaSuccess) e = cudaMemset(b->d_flag, 0, sizeof(int) * ndomains);
        b->bad_h.assign(ndomains, 0);
    }
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "mph_batch_create");
        free_batch(b);
        delete b;
        return rc;
    }
    int rc = build_walls(b);
    if (!rc && shifted(b->prec)) rc = build_row_chunks(b);
    if (rc) {
        free_batch(b);
        delete b;
        return rc;
    }
    *out = b;
    return MPH_OK;
}

int mph_batch_destroy(mph_batch* b) {
    if (!b) return MPH_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return MPH_OK;
}

int mph_batch_init_fields(mph_batch* b, int domain, double* rho, double* u) {
    if (!b || !rho || !u || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_init_fields: bad argument");
    const mph_desc& ds = b->descs[domain];
    const KParams& kp = b->params_h[domain];
    const long long N = kp.ncell;
    if (!b->d_rho) MPH_CK(cudaMalloc(&b->d_rho, sizeof(double) * b->max_cells), "batch rho");
    if (!b->d_u) MPH_CK(cudaMalloc(&b->d_u, sizeof(double) * 3 * b->max_cells), "batch u");
    MPH_CK(cudaMemcpyAsync(b->d_rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice, b->stream), "batch init rho");
    MPH_CK(cudaMemcpyAsync(b->d_u, u, sizeof(double) * ds.dim * N, cudaMemcpyHostToDevice, b->stream), "batch init u");
    void* base = static_cast<char*>(b->fa) + elem_of(b->prec) * b->offs_h[domain];
    MPH_CK(launch_init(b->prec, b->q, b->forced, base, b->d_rho, b->d_u, kp, b->stream), "batch init");
    if (b->forced) {
        MPH_CK(cudaMemcpyAsync(rho, b->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, b->stream), "batch init rho");
        MPH_CK(cudaMemcpyAsync(u, b->d_u, sizeof(double) * ds.dim * N, cudaMemcpyDeviceToHost, b->stream), "batch init u");
    }
    MPH_CK(cudaStreamSynchronize(b->stream), "batch init");
    b->time = 0.0;
    b->has_uprev = false;
    if (!b->bad_h.empty()) b->bad_h[domain] = 0;
    return b->prec == MPH_PREC_F16W ? check_flag(b) : MPH_OK;  // saturated stores of the new state
}

int mph_batch_init_fields_neq(mph_batch* b, int domain, const double* rho, const double* u) {
    if (!b || !rho || !u || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_init_fields_neq: bad argument");
    if (b->forced) return fail(MPH_ERR_UNSUPPORTED, "mph_batch_init_fields_neq: forced domains are not supported");
    const mph_desc& ds = b->descs[domain];
    const KParams& kp = b->params_h[domain];
    const long long N = kp.ncell;
    if (!b->d_rho) MPH_CK(cudaMalloc(&b->d_rho, sizeof(double) * b->max_cells), "batch rho");
    if (!b->d_u) MPH_CK(cudaMalloc(&b->d_u, sizeof(double) * 3 * b->max_cells), "batch u");
    MPH_CK(cudaMemcpyAsync(b->d_rho, rho, sizeof(double) * N, cudaMemcpyHostToDevice, b->stream), "batch init rho");
    MPH_CK(cudaMemcpyAsync(b->d_u, u, sizeof(double) * ds.dim * N, cudaMemcpyHostToDevice, b->stream), "batch init u");
    void* base = static_cast<char*>(b->fa) + elem_of(b->prec) * b->offs_h[domain];
    MPH_CK(launch_init_neq(b->prec, b->q, base, b->d_rho, b->d_u, kp, b->stream), "batch init");
    MPH_CK(cudaStreamSynchronize(b->stream), "batch init");
    b->time = 0.0;
    b->has_uprev = false;
    if (!b->bad_h.empty()) b->bad_h[domain] = 0;
    return b->prec == MPH_PREC_F16W ? check_flag(b) : MPH_OK;  // saturated stores of the new state
}

int mph_batch_advance(mph_batch* b, int nsteps) {
    if (!b || nsteps < 0) return fail(MPH_ERR_ARG, "mph_batch_advance: bad argument");
    int rc = advance_batch(b, nsteps);
    if (rc) return rc;
    MPH_CK(cudaStreamSynchronize(b->stream), "mph_batch_advance");
    return check_flag(b);
}

int mph_batch_advance_timed(mph_batch* b, int nsteps, float* ms) {
    if (!b || nsteps < 0 || !ms) return fail(MPH_ERR_ARG, "mph_batch_advance_timed: bad argument");
    int rc = autotune(b);
    if (!rc) rc = ensure_graph(b);
    if (rc) return rc;
    MPH_CK(cudaEventRecord(b->ev0, b->stream), "event");
    rc = advance_batch(b, nsteps);
    if (rc) return rc;
    MPH_CK(cudaEventRecord(b->ev1, b->stream), "event");
    MPH_CK(cudaEventSynchronize(b->ev1), "event sync");
    MPH_CK(cudaEventElapsedTime(ms, b->ev0, b->ev1), "event elapsed");
    return check_flag(b);
}

int mph_batch_advance_looped_timed(mph_batch* b, int nsteps, float* ms) {
    if (!b || nsteps < 0 || !ms) return fail(MPH_ERR_ARG, "mph_batch_advance_looped_timed: bad argument");
    MPH_CK(cudaEventRecord(b->ev0, b->stream), "event");
    const size_t es = elem_of(b->prec);
    for (int t = 0; t < nsteps; ++t) {
        for (int d = 0; d < b->ndom; ++d) {
            const KParams& kp = b->params_h[d];
            const void* in = static_cast<const char*>(b->fa) + es * b->offs_h[d];
            void* outp = static_cast<char*>(b->fb) + es * b->offs_h[d];
            cudaError_t e = cudaErrorInvalidValue;
            const KParams* pg = b->d_params + d;
            switch (b->prec) {
                case MPH_PREC_F64: e = launch_step_exact(b->q, b->forced, (const double*)in, (double*)outp, kp, pg, b->stream); break;
                case MPH_PREC_F64_FAST: e = launch_step_fast_f64(b->q, b->forced, (const double*)in, (double*)outp, kp, pg, b->stream); break;
                case MPH_PREC_F32: e = launch_step_fast_f32(b->q, b->forced, (const float*)in, (float*)outp, kp, pg, b->stream); break;
                case MPH_PREC_F16S: e = launch_step_fast_f16s(b->q, b->forced, in, outp, kp, pg, b->stream); break;
                case MPH_PREC_BF16S: e = launch_step_fast_bf16s(b->q, b->forced, in, outp, kp, pg, b->stream); break;
                case MPH_PREC_F16C: e = launch_step_fast_f16c(b->q, b->forced, in, outp, kp, pg, b->stream); break;
                case MPH_PREC_F16W: e = launch_step_fast_f16w(b->q, b->forced, in, outp, kp, pg, b->stream); break;
                case MPH_PREC_F64X:
                    e = launch_step_f64x(b->q, b->forced, (const long long*)in, (long long*)outp, kp, b->px_h[d], pg,
                                         b->d_kbb + (size_t)d * 27 * 27, b->d_flag + d, b->stream);
                    break;
            }
            if (e != cudaSuccess) return cuda_fail(e, "looped step launch");
        }
        std::swap(b->fa, b->fb);
    }
    b->time += nsteps;
    MPH_CK(cudaEventRecord(b->ev1, b->stream), "event");
    MPH_CK(cudaEventSynchronize(b->ev1), "event sync");
    MPH_CK(cudaEventElapsedTime(ms, b->ev0, b->ev1), "event elapsed");
    return check_flag(b);
}

int mph_batch_get_f(mph_batch* b, int domain, double* f) {
    if (!b || !f || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_get_f: bad argument");
    const KParams& kp = b->params_h[domain];
    const long long N = kp.ncell;
    const size_t es = elem_of(b->prec);
    void* base = static_cast<char*>(b->fa) + es * b->offs_h[domain];
    if (es == 8 && (b->prec == MPH_PREC_F64 || b->prec == MPH_PREC_F64_FAST)) {
        MPH_CK(cudaMemcpyAsync(f, base, sizeof(double) * b->q * N, cudaMemcpyDeviceToHost, b->stream), "batch get f");
    } else {
        if (!b->d_stage) MPH_CK(cudaMalloc(&b->d_stage, sizeof(double) * b->max_cells), "batch stage");
        for (int q = 0; q < b->q; ++q) {
            MPH_CK(launch_convert(b->prec, b->q, false, base, b->d_stage, q, N, b->stream), "batch convert");
            MPH_CK(cudaMemcpyAsync(f + (size_t)q * N, b->d_stage, sizeof(double) * N, cudaMemcpyDeviceToHost, b->stream),
                   "batch get f");
        }
    }
    MPH_CK(cudaStreamSynchronize(b->stream), "batch get f");
    return MPH_OK;
}

int mph_batch_set_f(mph_batch* b, int domain, const double* f) {
    if (!b || !f || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_set_f: bad argument");
    const KParams& kp = b->params_h[domain];
    const long long N = kp.ncell;
    const size_t es = elem_of(b->prec);
    void* base = static_cast<char*>(b->fa) + es * b->offs_h[domain];
    if (b->prec == MPH_PREC_F64 || b->prec == MPH_PREC_F64_FAST) {
        MPH_CK(cudaMemcpyAsync(base, f, sizeof(double) * b->q * N, cudaMemcpyHostToDevice, b->stream), "batch set f");
    } else {
        if (!b->d_stage) MPH_CK(cudaMalloc(&b->d_stage, sizeof(double) * b->max_cells), "batch stage");
        for (int q = 0; q < b->q; ++q) {
            MPH_CK(cudaMemcpyAsync(b->d_stage, f + (size_t)q * N, sizeof(double) * N, cudaMemcpyHostToDevice,
                                   b->stream), "batch set f");
            MPH_CK(launch_convert(b->prec, b->q, true, base, b->d_stage, q, N, b->stream,
                                  per_domain_flags(b->prec) ? b->d_flag + domain : nullptr),
                   "batch convert");
        }
    }
    MPH_CK(cudaStreamSynchronize(b->stream), "batch set f");
    b->has_uprev = false;
    if (!b->bad_h.empty()) b->bad_h[domain] = 0;
    return b->prec == MPH_PREC_F16W ? check_flag(b) : MPH_OK;
}

int mph_batch_moments(mph_batch* b, int domain, double* rho, double* u) {
    if (!b || !rho || !u || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_moments: bad argument");
    const KParams& kp = b->params_h[domain];
    const long long N = kp.ncell;
    if (!b->d_rho) MPH_CK(cudaMalloc(&b->d_rho, sizeof(double) * b->max_cells), "batch rho");
    if (!b->d_u) MPH_CK(cudaMalloc(&b->d_u, sizeof(double) * 3 * b->max_cells), "batch u");
    const void* base = static_cast<const char*>(b->fa) + elem_of(b->prec) * b->offs_h[domain];
    MPH_CK(launch_moments(b->prec, b->q, b->forced, base, b->d_rho, b->d_u, kp, b->d_params + domain, b->stream),
           "batch moments");
    MPH_CK(cudaMemcpyAsync(rho, b->d_rho, sizeof(double) * N, cudaMemcpyDeviceToHost, b->stream), "batch rho");
    MPH_CK(cudaMemcpyAsync(u, b->d_u, sizeof(double) * b->dim * N, cudaMemcpyDeviceToHost, b->stream), "batch u");
    MPH_CK(cudaStreamSynchronize(b->stream), "batch moments");
    return MPH_OK;
}

int mph_batch_set_obstacles(mph_batch* b, int domain, const unsigned char* mask) {
    if (!b || domain < 0 || domain >= b->ndom) return fail(MPH_ERR_ARG, "mph_batch_set_obstacles: bad argument");
    MPH_CK(cudaStreamSynchronize(b->stream), "mph_batch_set_obstacles");
    KParams& p = b->params_h[domain];
    if (!mask) {
        b->cls_h[domain].clear();
        p.cls = nullptr;
    } else {
        if (!b->d_cls) MPH_CK(cudaMalloc(&b->d_cls, b->total_cells), "batch obstacle classes");
        auto& cls = b->cls_h[domain];
        cls.assign(p.ncell, 0);
        build_cls(p, b->q, mask, cls.data());
        unsigned char* dst = b->d_cls + b->coffs_h[domain];
        MPH_CK(cudaMemcpy(dst, cls.data(), p.ncell, cudaMemcpyHostToDevice), "batch obstacle classes");
        p.cls = dst;
    }
    MPH_CK(cudaMemcpy(b->d_params + domain, &p, sizeof(KParams), cudaMemcpyHostToDevice), "batch parameters");
    int rc = build_walls(b);
    if (rc) return rc;
    drop_graphs(b);  // the captured steps name the old wall list
    return MPH_OK;
}

int mph_batch_residual(mph_batch* b, double* out) {
    if (!b || !out) return fail(MPH_ERR_ARG, "mph_batch_residual: NULL argument");
    int rc = ensure_chunks(b, 0);  // K = 1 chunk list, independent of the tuned K
    if (rc) return rc;
    if (!b->d_uprev) {
        MPH_CK(cudaMalloc(&b->d_uprev, sizeof(double) * b->dim * b->total_cells), "batch residual field");
        MPH_CK(cudaMalloc(&b->d_coffs, sizeof(long long) * b->ndom), "batch residual offsets");
        MPH_CK(cudaMemcpy(b->d_coffs, b->coffs_h.data(), sizeof(long long) * b->ndom, cudaMemcpyHostToDevice),
               "batch residual offsets");
        MPH_CK(cudaMalloc(&b->d_rpart, sizeof(double) * 2 * b->nchunks[0]), "batch residual partials");
        MPH_CK(cudaMalloc(&b->d_rout, sizeof(double) * 2 * b->ndom), "batch residual sums");
    }
    MPH_CK(launch_batch_residual(b->prec, b->q, b->fa, b->d_chunks[0], b->nchunks[0], kCells[0], b->d_params,
                                 b->d_offs, b->d_coffs, b->d_uprev, !b->has_uprev, b->d_rpart, b->d_chunk_first[0],
                                 b->ndom, b->d_rout, b->stream),
           "batch residual");
    std::vector<double> sums(2 * b->ndom);
    MPH_CK(cudaMemcpyAsync(sums.data(), b->d_rout, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, b->stream),
           "batch residual download");
    MPH_CK(cudaStreamSynchronize(b->stream), "batch residual");
    for (int d = 0; d < b->ndom; ++d) {
        const double s0 = sums[2 * d], s1 = sums[2 * d + 1];
        out[2 * d + 1] = std::sqrt(s1);
        out[2 * d] = relative_change(s0, s1, b->has_uprev);
        // a fixed-point domain that left the representable range holds no
        // meaningful populations: report it as diverged
        if (!b->bad_h.empty() && b->bad_h[d]) out[2 * d] = out[2 * d + 1] = std::nan("");
    }
    b->has_uprev = true;
    return MPH_OK;
}

int mph_batch_range_flags(const mph_batch* b, int* flags) {
    if (!b || !flags) return fail(MPH_ERR_ARG, "mph_batch_range_flags: NULL argument");
    for (int d = 0; d < b->ndom; ++d) flags[d] = b->bad_h.empty() ? 0 : b->bad_h[d];
    return MPH_OK;
}

int mph_batch_info(const mph_batch* b, long long* total_cells, int* cells_per_thread, int* nchunks, int* persistent) {
    if (!b) return fail(MPH_ERR_ARG, "mph_batch_info: NULL batch");
    if (total_cells) *total_cells = b->total_cells;
    const bool staged = b->k_idx == kBulkCand;
    if (cells_per_thread) *cells_per_thread = b->k_idx >= 0 ? (staged ? 2 : kCells[b->k_idx % 3]) : 0;
    if (nchunks) *nchunks = b->k_idx >= 0 ? (staged ? b->nrchunks : b->nchunks[b->k_idx % 3]) : 0;
    if (persistent) *persistent = b->k_idx >= 3 ? 1 : 0;
    return MPH_OK;
}

}  // extern "C"
