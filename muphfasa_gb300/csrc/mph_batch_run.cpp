// mph_batch_run.cpp -- batch runner over the C ABI: many independent
// domains, each described by one of the reference's inputs files, advanced
// together by the batched kernel (mph_batch_*), each domain with the loop of
// the reference's main.cpp:14-38 (steps 0 .. sim.max_step, the sim.stop_time
// check, a plot directory every amr.plot_int steps).
//
//   mph_batch_run <inputs file> [<inputs file> ...] [key=value ...]
//
// Every key=value override applies to every domain.  Extra keys:
//   mph.precision  f64 | f64_fast | f64x | f32 | f16s | bf16s | f16c | f16w
//                  (default f64, the reference's arithmetic; one precision
//                  for the batch).  With f64x (f16w) a domain whose
//                  populations leave the fixed-point (16-bit) range stops
//                  there and is reported "diverged"; the others go on.
//   mph.device     CUDA device (default 0)
//   mph.tol        > 0: a domain also stops once the steady-state residual
//                  (relative change of its velocity over mph.check_every
//                  steps, FP64) falls below mph.tol
//   mph.check_every  steps between residual checks (default 100)
//   mph.out        output root (default "."): domain i writes its plot
//                  directories and a final one under <mph.out>/domain<i:04d>/
//
// All domains share lattice, precision and forcing flag (mph_batch_create).
// Domains that have stopped keep being stepped with the others; their
// outputs are frozen at their own last step.  One summary line per domain
// goes to standard output.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "driver_util.h"
#include "mph.h"

using namespace drv;

namespace {

struct Domain {
    std::string inputs;
    mph_desc d;
    mph_run_info info;
    int last = 0;         // last loop step (max_step, or the stop-time bound)
    int done_step = -1;   // loop step at which the domain stopped (-1: running)
    double residual = NAN;
    bool diverged = false;  // left the storage's range (f64x, f16w)
    std::string dir, plot_prefix;
};

// Loop step after which domain m stops by max_step / stop_time
// (main.cpp: iterate while the lattice time t = step does not exceed the
// stop time).
int last_step(const mph_run_info& info) {
    int last = info.max_step;
    if (info.stop_time > 0) {
        const double stop_lat = info.stop_time / info.dt;
        if (stop_lat < last) last = (int)std::floor(stop_lat);
    }
    return last;
}

}  // namespace

int main(int argc, char** argv) {
    program() = "mph_batch_run";
    std::vector<std::string> files;
    std::vector<const char*> over;
    for (int i = 1; i < argc; ++i) {
        if (std::strchr(argv[i], '=')) over.push_back(argv[i]);
        else files.push_back(argv[i]);
    }
    if (files.empty()) {
        std::cerr << "usage: mph_batch_run <inputs file> [<inputs file> ...] [key=value ...]\n";
        return 2;
    }
    std::vector<Domain> dom(files.size());
    std::string prec_name, out_root;
    int prec = -1, device = 0, check_every = 100;
    double tol = 0.0;
    for (size_t i = 0; i < files.size(); ++i) {
        mph_inputs* in = nullptr;
        ck(mph_inputs_load(files[i].c_str(), (int)over.size(), over.data(), &in), "inputs");
        if (i == 0) {
            prec_name = get(in, "mph.precision", "f64");
            prec = precision_code(prec_name);
            if (prec < 0) die("mph.precision must be one of f64 f64_fast f64x f32 f16s bf16s f16c f16w");
            device = std::atoi(get(in, "mph.device", "0").c_str());
            tol = std::atof(get(in, "mph.tol", "0").c_str());
            check_every = std::atoi(get(in, "mph.check_every", "100").c_str());
            if (check_every < 1) die("mph.check_every must be >= 1");
            out_root = get(in, "mph.out", ".");
            ck(mph_set_device(device), "device");
        }
        Domain& m = dom[i];
        m.inputs = files[i];
        ck(mph_inputs_derive(in, prec, &m.d, &m.info), "inputs");
        m.last = last_step(m.info);
        m.plot_prefix = get(in, "amr.plot_file", "plt");
        std::ostringstream ss;
        ss << out_root << "/domain" << std::setw(4) << std::setfill('0') << i;
        m.dir = ss.str();
        mph_inputs_free(in);
    }
    make_dir(out_root);
    std::vector<mph_desc> descs;
    for (const Domain& m : dom) descs.push_back(m.d);
    mph_batch* b = nullptr;
    ck(mph_batch_create((int)descs.size(), descs.data(), &b), "batch");
    for (size_t i = 0; i < dom.size(); ++i) {
        const long long N = cells(dom[i].d);
        std::vector<double> rho(N, 1.0), u((size_t)dom[i].d.dim * N, 0.0);  // initData: quiescent start
        ck(mph_batch_init_fields(b, (int)i, rho.data(), u.data()), "initialize");
        make_dir(dom[i].dir);
    }

    auto write = [&](size_t i, int step, const std::string& dir) {
        const Domain& m = dom[i];
        const long long N = cells(m.d);
        std::vector<double> rho(N), u((size_t)m.d.dim * N);
        ck(mph_batch_moments(b, (int)i, rho.data(), u.data()), "moments");
        write_plot(dir, rho, u, m.d, m.info, (double)(step + 1), step);
    };

    // The loop of main.cpp, over all domains at once: after loop step s every
    // domain has advanced s + 1 times.  The batch advances in one call up to
    // the next step at which some running domain plots, checks or stops.
    int step = -1;  // last loop step completed
    std::vector<double> res(2 * dom.size());
    if (tol > 0) ck(mph_batch_residual(b, res.data()), "residual");  // reference velocity
    for (;;) {
        int next = INT_MAX;
        for (const Domain& m : dom) {
            if (m.done_step >= 0) continue;
            next = std::min(next, m.last);
            const int pi = m.info.plot_int;
            if (pi > 0) next = std::min(next, (step + 1 + pi - 1) / pi * pi);
            if (tol > 0) next = std::min(next, (step + 1 + check_every) / check_every * check_every - 1);
        }
        if (next == INT_MAX) break;
        const int rc = mph_batch_advance(b, next - step);
        if (rc == MPH_ERR_NONFINITE && (prec == MPH_PREC_F64X || prec == MPH_PREC_F16W)) {
            // domains that left the storage's range stop where they are
            std::vector<int> flags(dom.size(), 0);
            ck(mph_batch_range_flags(b, flags.data()), "range flags");
            for (size_t i = 0; i < dom.size(); ++i)
                if (flags[i] && dom[i].done_step < 0) {
                    dom[i].done_step = next;
                    dom[i].diverged = true;
                }
        } else {
            ck(rc, "advance");
        }
        step = next;
        if (tol > 0 && (step + 1) % check_every == 0) ck(mph_batch_residual(b, res.data()), "residual");
        for (size_t i = 0; i < dom.size(); ++i) {
            Domain& m = dom[i];
            if (m.done_step >= 0) continue;
            if (m.info.plot_int > 0 && step % m.info.plot_int == 0) {
                write(i, step, m.dir + "/" + numbered(m.plot_prefix, step));
            }
            bool stop = step >= m.last;
            if (tol > 0 && (step + 1) % check_every == 0) {
                m.residual = res[2 * i];
                if (m.residual < tol) stop = true;
            }
            if (stop) {
                m.done_step = step;
                write(i, step, m.dir + "/final");
            }
        }
    }
    for (size_t i = 0; i < dom.size(); ++i) {
        const Domain& m = dom[i];
        if (m.diverged) {
            std::cout << "domain " << i << " " << m.inputs << ": diverged (left the storage's range) by step "
                      << m.done_step + 1 << "\n";
            continue;
        }
        std::cout << "domain " << i << " " << m.inputs << ": steps " << m.done_step + 1 << " residual "
                  << std::setprecision(6) << m.residual << (tol > 0 && m.residual < tol ? " converged" : "")
                  << " -> " << m.dir << "/final\n";
    }
    ck(mph_batch_destroy(b), "batch");
    return 0;
}
