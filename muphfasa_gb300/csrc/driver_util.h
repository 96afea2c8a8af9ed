// driver_util.h -- helpers shared by the host drivers (mph_run.cpp,
// mph_batch_run.cpp): inputs lookups, numbered directories, NumPy output and
// the plot directory (density and velocity in physical units,
// SimulationSetup.cpp:169-198 / Units.cpp:185-199).
#pragma once

#include <sys/stat.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "mph.h"

namespace drv {

inline const char*& program() {
    static const char* name = "mph_run";
    return name;
}

[[noreturn]] inline void die(const std::string& what) {
    std::cerr << program() << ": " << what << "\n";
    std::exit(1);
}

inline void ck(int rc, const char* what) {
    if (rc != MPH_OK) die(std::string(what) + ": " + mph_last_error());
}

// A single-token value of an inputs key, or dflt.
inline std::string get(const mph_inputs* in, const char* key, const std::string& dflt) {
    char buf[4096];
    if (mph_inputs_get(in, key, buf, sizeof buf) != MPH_OK) return dflt;
    std::string s(buf);
    const size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// mph.precision names of the storage precisions.
inline int precision_code(const std::string& name) {
    const char* names[] = {"f64", "f64_fast", "f32", "f16s", "bf16s", "f64x", "f16c", "f16w"};
    const int precs[] = {MPH_PREC_F64, MPH_PREC_F64_FAST, MPH_PREC_F32, MPH_PREC_F16S, MPH_PREC_BF16S, MPH_PREC_F64X,
                         MPH_PREC_F16C, MPH_PREC_F16W};
    for (int i = 0; i < 8; ++i)
        if (name == names[i]) return precs[i];
    return -1;
}

inline std::string numbered(const std::string& prefix, int step) {
    std::ostringstream ss;
    ss << prefix << std::setw(7) << std::setfill('0') << step;
    return ss.str();
}

inline void make_dir(const std::string& d) {
    if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) die("cannot create directory " + d);
}

inline std::string domain_box(const mph_desc& d) {
    std::ostringstream ss;
    if (d.dim == 2) ss << "((0,0) (" << d.n[0] - 1 << "," << d.n[1] - 1 << ") (0,0))";
    else ss << "((0,0,0) (" << d.n[0] - 1 << "," << d.n[1] - 1 << "," << d.n[2] - 1 << ") (0,0,0))";
    return ss.str();
}

inline long long cells(const mph_desc& d) { return (long long)d.n[0] * d.n[1] * (d.dim == 3 ? d.n[2] : 1); }

// One field as a .npy file, shape (nz,) ny, nx.
inline void write_npy(const std::string& path, const double* v, const mph_desc& d) {
    std::ostringstream hdr;
    hdr << "{'descr': '<f8', 'fortran_order': False, 'shape': (";
    if (d.dim == 3) hdr << d.n[2] << ", ";
    hdr << d.n[1] << ", " << d.n[0] << "), }";
    std::string h = hdr.str();
    const size_t total = 10 + h.size() + 1;
    h.append((64 - total % 64) % 64, ' ');
    h.push_back('\n');
    std::ofstream f(path, std::ios::binary);
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    f.write(reinterpret_cast<const char*>(magic), 8);
    const unsigned short len = (unsigned short)h.size();
    const unsigned char le[2] = {(unsigned char)(len & 0xff), (unsigned char)(len >> 8)};
    f.write(reinterpret_cast<const char*>(le), 2);
    f.write(h.data(), (std::streamsize)h.size());
    f.write(reinterpret_cast<const char*>(v), (std::streamsize)(cells(d) * sizeof(double)));
    if (!f) die("cannot write " + path);
}

// A plot directory from lattice moments (rho, u: valid cells, u component
// slowest): density = rho ref_density, velocity = u dx / dt, a Header with
// the variable names, dimension, physical time, step and domain box.  rho
// and u are scaled in place.
inline void write_plot(const std::string& dir, std::vector<double>& rho, std::vector<double>& u, const mph_desc& d,
                       const mph_run_info& info, double t_lattice, int step) {
    make_dir(dir);
    const long long N = cells(d);
    for (auto& r : rho) r *= info.ref_density;
    for (auto& v : u) v *= info.dx / info.dt;
    write_npy(dir + "/density.npy", rho.data(), d);
    const char* vn[3] = {"vx", "vy", "vz"};
    for (int a = 0; a < d.dim; ++a) write_npy(dir + "/" + vn[a] + ".npy", u.data() + (size_t)a * N, d);
    std::ofstream h(dir + "/Header");
    h << "muphfasa_gb300_plotfile_v1\n" << (d.dim + 1) << "\ndensity\n";
    for (int a = 0; a < d.dim; ++a) h << vn[a] << "\n";
    h << d.dim << "\n" << std::setprecision(17) << t_lattice * info.dt << "\n" << step << "\n" << domain_box(d) << "\n";
    if (!h) die("cannot write " + dir + "/Header");
}

}  // namespace drv
