// mph_run.cpp -- host driver over the C ABI, the counterpart of the
// reference's main.cpp:14-38 (InputParser -> makeSimulation -> initialize ->
// for step = startStep .. max_step: stop-time check, advance, writeOutput).
//
//   mph_run <inputs file> [key=value ...]
//
// Reads the reference's inputs keys; two extra keys select this build's
// options: mph.precision (f64 | f64_fast | f32 | f16s | bf16s | f64x | f16c |
// f16w, default f64, the reference's arithmetic) and mph.device (default 0).
//
// Output (SimulationSetup.cpp:169-198):
//   * every amr.plot_int steps a plot directory <amr.plot_file><step:07d>
//     with density and velocity in physical units (rho * ref_density,
//     u * dx / dt, Units.cpp:185-199), one NumPy .npy file per variable
//     (shape (nz,) ny, nx) and a text Header; the AMReX plotfile format itself
//     is AMReX-defined and not reproduced;
//   * every amr.chk_int steps a checkpoint <amr.check_file><step:07d>: the
//     reference's Header lines (Checkpoint.cpp:36-44: version, step, time,
//     domain box, component count, ghost vector; version string of this
//     build) plus a line naming the storage precision, the populations as
//     raw little-endian FP64 in valid-cell SoA order (x fastest, population
//     slowest, f.f64) in place of VisMF, and the handle's own storage
//     (state.raw) so that every precision resumes bit for bit;
//   * amr.restart = <checkpoint directory> resumes from such a checkpoint
//     with step + 1 (SimulationSetup.cpp:107-117), bit for bit.
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "driver_util.h"
#include "mph.h"

using namespace drv;

namespace {
constexpr const char* kCheckpointVersion = "muphfasa_gb300_checkpoint_v1";
}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: mph_run <inputs file> [key=value ...]\n";
        return 2;
    }
    mph_inputs* in = nullptr;
    ck(mph_inputs_load(argv[1], argc - 2, const_cast<const char* const*>(argv + 2), &in), "inputs");
    const std::string prec_name = get(in, "mph.precision", "f64");
    const int prec = precision_code(prec_name);
    if (prec < 0) die("mph.precision must be one of f64 f64_fast f32 f16s bf16s f64x f16c f16w");
    ck(mph_set_device(std::atoi(get(in, "mph.device", "0").c_str())), "device");

    mph_desc d;
    mph_run_info info;
    ck(mph_inputs_derive(in, prec, &d, &info), "inputs");
    mph_sim* sim = nullptr;
    ck(mph_create(&d, &sim), "create");
    const long long N = cells(d);
    const std::string plot_prefix = get(in, "amr.plot_file", "plt");
    const std::string chk_prefix = get(in, "amr.check_file", "chk");
    const std::string restart = get(in, "amr.restart", "");

    int start = 0;
    if (restart.empty()) {
        std::vector<double> rho(N, 1.0), u((size_t)d.dim * N, 0.0);  // initData: quiescent start
        ck(mph_init_fields(sim, rho.data(), u.data()), "initialize");
    } else {
        std::ifstream hdr(restart + "/Header");
        if (!hdr) die("no Header file found in " + restart);
        std::string version, domain, ngrow, stored;
        int step = 0, ncomp = 0;
        double time = 0.0;
        hdr >> version >> step >> time >> std::ws;
        std::getline(hdr, domain);
        hdr >> ncomp >> ngrow;
        if (version != kCheckpointVersion) die("unrecognized checkpoint version \"" + version + "\" in " + restart);
        if (!hdr || domain != domain_box(d) || ncomp != d.q) die("checkpoint " + restart + " does not match the domain");
        hdr >> stored;  // "mph.precision=<name>" (optional)
        long long nbytes = 0;
        ck(mph_state_bytes(sim, &nbytes), "restart");
        std::ifstream raw(restart + "/state.raw", std::ios::binary);
        if (stored == "mph.precision=" + prec_name && raw) {
            std::vector<unsigned char> st((size_t)nbytes);
            raw.read(reinterpret_cast<char*>(st.data()), (std::streamsize)nbytes);
            if (!raw) die("short state payload in " + restart);
            ck(mph_set_state(sim, st.data(), nbytes), "restart");
        } else {
            std::vector<double> f((size_t)d.q * N);
            std::ifstream fb(restart + "/f.f64", std::ios::binary);
            fb.read(reinterpret_cast<char*>(f.data()), (std::streamsize)(f.size() * sizeof(double)));
            if (!fb) die("short checkpoint payload in " + restart);
            ck(mph_set_f(sim, f.data()), "restart");
        }
        ck(mph_set_time(sim, time), "restart");
        start = step + 1;
    }

    const double stop_lat = info.stop_time > 0 ? info.stop_time / info.dt : 0.0;  // toLatticeTime
    std::vector<double> rho(N), u((size_t)d.dim * N), f;
    for (int step = start; step <= info.max_step; ++step) {
        double t = 0.0;
        ck(mph_time(sim, &t), "time");
        if (stop_lat > 0 && stop_lat < t) break;
        ck(mph_advance(sim, 1), "advance");
        ck(mph_time(sim, &t), "time");
        if (info.plot_int > 0 && step % info.plot_int == 0) {
            ck(mph_update_macroscopic(sim, rho.data(), u.data()), "moments");
            const std::string dir = numbered(plot_prefix, step);
            write_plot(dir, rho, u, d, info, t, step);
            std::cout << "Plotfile: wrote " << dir << "  step=" << step << "  time=" << t * info.dt << "\n";
        }
        if (info.chk_int > 0 && step % info.chk_int == 0) {
            const std::string dir = numbered(chk_prefix, step);
            make_dir(dir);
            f.resize((size_t)d.q * N);
            ck(mph_get_f(sim, f.data()), "checkpoint");
            std::ofstream h(dir + "/Header");
            h << kCheckpointVersion << "\n" << step << "\n" << std::setprecision(17) << t << "\n" << domain_box(d)
              << "\n" << d.q << "\n" << (d.dim == 2 ? "(0,0)" : "(0,0,0)") << "\nmph.precision=" << prec_name << "\n";
            std::ofstream fb(dir + "/f.f64", std::ios::binary);
            fb.write(reinterpret_cast<const char*>(f.data()), (std::streamsize)(f.size() * sizeof(double)));
            long long nbytes = 0;
            ck(mph_state_bytes(sim, &nbytes), "checkpoint");
            std::vector<unsigned char> st((size_t)nbytes);
            ck(mph_get_state(sim, st.data(), nbytes), "checkpoint");
            std::ofstream rb(dir + "/state.raw", std::ios::binary);
            rb.write(reinterpret_cast<const char*>(st.data()), (std::streamsize)nbytes);
            if (!fb || !h || !rb) die("cannot write checkpoint " + dir);
            std::cout << "Checkpoint: wrote " << dir << "  step=" << step << "  time=" << t << "\n";
        }
    }
    mph_destroy(sim);
    mph_inputs_free(in);
    return 0;
}
