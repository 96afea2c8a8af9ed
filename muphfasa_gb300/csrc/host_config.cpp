// host_config.cpp -- the host side of the step's configuration: a
// ParmParse-subset inputs reader, the InputParser accessors with their
// defaults, the physical-to-lattice unit converter and the boundary-condition
// resolution table.  Compiled with -ffp-contract=off so that the derived
// lattice quantities (omega, force, face velocities) carry the same bits as
// the reference's, which feed the bit-exact kernels.
#include "mph_internal.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace mph {

namespace {
thread_local std::string g_last_error;

enum { BC_MOVING = 0, BC_NOSLIP = 1, BC_INFLOW = 2, BC_OUTFLOW = 3, BC_PRESSURE = 4, BC_PERIODIC = 5 };
}  // namespace

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
void clear_error() { g_last_error.clear(); }

bool lattice_ok(int dim, int q) {
    return (dim == 2 && q == 9) || (dim == 3 && (q == 15 || q == 19 || q == 27));
}

const Def* Inputs::find(const std::string& key) const {
    for (auto it = defs.rbegin(); it != defs.rend(); ++it)
        if (it->key == key) return &*it;
    return nullptr;
}

namespace {

// Tokenizer of the ParmParse text format: '#' starts a comment to the end of
// the line, '=' is a token of its own, "..." is one token, and a token
// followed by '=' starts a new definition whose values run up to the next
// such key.
int tokenize(const std::string& text, std::vector<std::string>& toks) {
    size_t i = 0, n = text.size();
    while (i < n) {
        const char c = text[i];
        if (c == '#') {
            while (i < n && text[i] != '\n') ++i;
        } else if (std::isspace((unsigned char)c)) {
            ++i;
        } else if (c == '=') {
            toks.emplace_back("=");
            ++i;
        } else if (c == '"') {
            size_t j = i + 1;
            while (j < n && text[j] != '"') ++j;
            if (j >= n) return fail(MPH_ERR_PARSE, "inputs: unterminated quoted string");
            toks.emplace_back(text.substr(i + 1, j - i - 1));
            i = j + 1;
        } else {
            size_t j = i;
            while (j < n && !std::isspace((unsigned char)text[j]) && text[j] != '=' && text[j] != '#') ++j;
            toks.emplace_back(text.substr(i, j - i));
            i = j;
        }
    }
    return MPH_OK;
}

int parse_defs(const std::string& text, Inputs& in) {
    std::vector<std::string> t;
    int rc = tokenize(text, t);
    if (rc) return rc;
    size_t i = 0;
    while (i < t.size()) {
        if (i + 1 >= t.size() || t[i + 1] != "=" || t[i] == "=")
            return fail(MPH_ERR_PARSE, "inputs: expected 'key = value...' near token '" + t[i] + "'");
        Def d;
        d.key = t[i];
        i += 2;
        while (i < t.size() && t[i] != "=" && !(i + 1 < t.size() && t[i + 1] == "=")) d.vals.push_back(t[i++]);
        in.defs.push_back(std::move(d));
    }
    return MPH_OK;
}

bool to_double(const std::string& s, double& v) {
    if (s.empty()) return false;
    char* end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

bool to_int(const std::string& s, int& v) {
    if (s.empty()) return false;
    char* end = nullptr;
    long x = std::strtol(s.c_str(), &end, 10);
    if (!end || *end != '\0') return false;
    v = (int)x;
    return true;
}

// ParmParse-like typed accessors.  query*: absent -> keep default.
// get*: absent -> error.
struct PP {
    const Inputs& in;
    std::string prefix;
    std::string full(const char* name) const { return prefix + "." + name; }

    int query_str(const char* name, std::string& v, bool& found) const {
        const Def* d = in.find(full(name));
        found = d != nullptr;
        if (!d) return MPH_OK;
        if (d->vals.empty()) return fail(MPH_ERR_PARSE, "inputs: " + full(name) + " has no value");
        v = d->vals[0];
        return MPH_OK;
    }
    int query_double(const char* name, double& v, bool& found) const {
        std::string s;
        int rc = query_str(name, s, found);
        if (rc || !found) return rc;
        if (!to_double(s, v)) return fail(MPH_ERR_PARSE, "inputs: " + full(name) + " is not a number: " + s);
        return MPH_OK;
    }
    int query_int(const char* name, int& v, bool& found) const {
        std::string s;
        int rc = query_str(name, s, found);
        if (rc || !found) return rc;
        if (!to_int(s, v)) return fail(MPH_ERR_PARSE, "inputs: " + full(name) + " is not an integer: " + s);
        return MPH_OK;
    }
    int query_arr(const char* name, std::vector<std::string>& v) const {
        const Def* d = in.find(full(name));
        v.clear();
        if (d) v = d->vals;
        return MPH_OK;
    }
    int query_darr(const char* name, std::vector<double>& v) const {
        std::vector<std::string> s;
        query_arr(name, s);
        v.clear();
        for (auto& x : s) {
            double y;
            if (!to_double(x, y)) return fail(MPH_ERR_PARSE, "inputs: " + full(name) + " has a non-number: " + x);
            v.push_back(y);
        }
        return MPH_OK;
    }
    // getarr(name, v, 0, n): at least n values required, the first n taken.
    int get_darr(const char* name, std::vector<double>& v, int n) const {
        if (!in.find(full(name))) return fail(MPH_ERR_PARSE, "inputs: missing required key " + full(name));
        int rc = query_darr(name, v);
        if (rc) return rc;
        if ((int)v.size() < n) return fail(MPH_ERR_PARSE, "inputs: " + full(name) + " needs " + std::to_string(n) + " values");
        v.resize(n);
        return MPH_OK;
    }
};

int bc_code(const std::string& name, int& code) {
    if (name == "MovingWall") code = BC_MOVING;
    else if (name == "NoSlip") code = BC_NOSLIP;
    else if (name == "Inflow") code = BC_INFLOW;
    else if (name == "Outflow") code = BC_OUTFLOW;
    else if (name == "PressureOutlet") code = BC_PRESSURE;
    else if (name == "Periodic") code = BC_PERIODIC;
    else
        return fail(MPH_ERR_CONFIG, "unrecognized BC name \"" + name +
                                        "\" (expected MovingWall, NoSlip, Inflow, Outflow, PressureOutlet or Periodic)");
    return MPH_OK;
}

// hasConflictingBC (BoundaryConditions.cpp:37-57): at most one of
// Inflow/Outflow/PressureOutlet, and at most one MovingWall, per edge/corner.
bool conflicting(const int* t, int nt) {
    int in = 0, out = 0, pr = 0, moving = 0;
    for (int a = 0; a < nt; ++a) {
        in |= t[a] == BC_INFLOW;
        out |= t[a] == BC_OUTFLOW;
        pr |= t[a] == BC_PRESSURE;
        moving += t[a] == BC_MOVING;
    }
    return in + out + pr > 1 || moving > 1;
}

// bcRank (BoundaryConditions.H:82-92).
int rank_of(int t) {
    switch (t) {
        case BC_NOSLIP: return 3;
        case BC_MOVING: return 2;
        case BC_INFLOW: return 1;
        case BC_OUTFLOW:
        case BC_PRESSURE: return 0;
        default: return -1;
    }
}

}  // namespace

// BCManager::finalize + resolveBC (BoundaryConditions.cpp:59-155): for every
// ghost class (code_d in {-1,0,1}, periodic faces skipped) the highest-ranked
// touching face type wins and rho/U are averaged over faces of that type.
int resolve_table(const mph_desc& d, mph_resolved_bc* table) {
    if (!lattice_ok(d.dim, d.q)) return fail(MPH_ERR_ARG, "unsupported lattice (dim, q)");
    for (int f = 0; f < 2 * d.dim; ++f)
        if (d.face_type[f] < 0 || d.face_type[f] > BC_PERIODIC) return fail(MPH_ERR_ARG, "bad face_type");
    for (int dir = 0; dir < d.dim; ++dir)
        if (d.face_type[2 * dir + 1] == BC_PERIODIC && d.face_type[2 * dir] != BC_PERIODIC)
            return fail(MPH_ERR_CONFIG, "bc input requests \"Periodic\" on a face whose direction is not periodic");
    for (int idx = 0; idx < 27; ++idx) {
        table[idx].type = BC_PERIODIC;
        table[idx].rho = 1.0;
        table[idx].U[0] = table[idx].U[1] = table[idx].U[2] = 0.0;
    }
    int total = 1;
    for (int dd = 0; dd < d.dim; ++dd) total *= 3;
    for (int idx = 0; idx < total; ++idx) {
        int code[3] = {0, 0, 0}, tmp = idx;
        for (int dd = 0; dd < d.dim; ++dd) { code[dd] = tmp % 3 - 1; tmp /= 3; }
        int ft[3], fidx[3], nf = 0;
        for (int dd = 0; dd < d.dim; ++dd) {
            if (code[dd] == 0) continue;
            const int fi = 2 * dd + (code[dd] < 0 ? 0 : 1);
            if (d.face_type[fi] == BC_PERIODIC) continue;
            ft[nf] = d.face_type[fi];
            fidx[nf] = fi;
            ++nf;
        }
        if (nf == 0) continue;
        if (conflicting(ft, nf)) {
            static const char* nm[6] = {"xlo", "xhi", "ylo", "yhi", "zlo", "zhi"};
            std::string msg = "resolveBC: conflicting boundary conditions at the same edge/corner (faces:";
            for (int a = 0; a < nf; ++a) msg += std::string(" ") + nm[fidx[a]];
            return fail(MPH_ERR_CONFIG, msg + ")");
        }
        int max_rank = -1;
        for (int a = 0; a < nf; ++a) max_rank = rank_of(ft[a]) > max_rank ? rank_of(ft[a]) : max_rank;
        int winner = 0;
        for (int a = 0; a < nf; ++a)
            if (rank_of(ft[a]) == max_rank) { winner = ft[a]; break; }
        double sum_rho = 0;
        double sum_U[3] = {0., 0., 0.};
        int count = 0;
        for (int a = 0; a < nf; ++a) {
            if (ft[a] != winner) continue;
            sum_rho += d.face_rho[fidx[a]];
            for (int c = 0; c < d.dim; ++c) sum_U[c] += d.face_U[fidx[a]][c];
            ++count;
        }
        table[idx].type = winner;
        table[idx].rho = sum_rho / count;
        for (int c = 0; c < d.dim; ++c) table[idx].U[c] = sum_U[c] / count;
    }
    return MPH_OK;
}

}  // namespace mph

using namespace mph;

struct mph_inputs {
    Inputs in;
};

extern "C" {

const char* mph_last_error(void) { return g_last_error.c_str(); }
int mph_abi_version(void) { return MPH_ABI_VERSION; }

static int load_common(const std::string& text, int noverrides, const char* const* overrides, mph_inputs** out) {
    if (!out) return fail(MPH_ERR_ARG, "mph_inputs_load: out is NULL");
    *out = nullptr;
    auto* p = new mph_inputs();
    int rc = parse_defs(text, p->in);
    for (int a = 0; rc == MPH_OK && a < noverrides; ++a) {
        if (!overrides || !overrides[a]) { rc = fail(MPH_ERR_ARG, "override is NULL"); break; }
        rc = parse_defs(overrides[a], p->in);
    }
    if (rc) { delete p; return rc; }
    *out = p;
    return MPH_OK;
}

int mph_inputs_load(const char* path, int noverrides, const char* const* overrides, mph_inputs** out) {
    std::string text;
    if (path) {
        std::ifstream f(path);
        if (!f) return fail(MPH_ERR_PARSE, std::string("cannot open inputs file ") + path);
        std::stringstream ss;
        ss << f.rdbuf();
        text = ss.str();
    }
    return load_common(text, noverrides, overrides, out);
}

int mph_inputs_parse_string(const char* text, int noverrides, const char* const* overrides, mph_inputs** out) {
    return load_common(text ? std::string(text) : std::string(), noverrides, overrides, out);
}

void mph_inputs_free(mph_inputs* in) { delete in; }

int mph_inputs_get(const mph_inputs* in, const char* key, char* buf, size_t buflen) {
    if (!in || !key || !buf || buflen == 0) return fail(MPH_ERR_ARG, "mph_inputs_get: bad argument");
    const Def* d = in->in.find(key);
    if (!d) return fail(MPH_ERR_ARG, std::string("key not defined: ") + key);
    std::string s;
    for (size_t a = 0; a < d->vals.size(); ++a) s += (a ? " " : "") + d->vals[a];
    if (s.size() + 1 > buflen) return fail(MPH_ERR_ARG, "mph_inputs_get: buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return MPH_OK;
}

int mph_resolve_bc(const mph_desc* desc, mph_resolved_bc* table) {
    if (!desc || !table) return fail(MPH_ERR_ARG, "mph_resolve_bc: NULL argument");
    return resolve_table(*desc, table);
}

// SimulationImpl's constructor (SimulationSetup.cpp:32-89) and buildBCManager
// (SimulationSetup.cpp:237-299) over the InputParser accessors
// (InputParser.cpp:75-323) and the UnitConverter (Units.cpp:20-183).
int mph_inputs_derive(const mph_inputs* inp, int precision, mph_desc* desc, mph_run_info* info) {
    if (!inp || !desc) return fail(MPH_ERR_ARG, "mph_inputs_derive: NULL argument");
    const Inputs& in = inp->in;
    bool found = false;
    int rc;
    mph_desc d;
    std::memset(&d, 0, sizeof(d));
    mph_run_info ri;
    std::memset(&ri, 0, sizeof(ri));

    // lbm.lattice_type (default D3Q19) and lbm.collision_model (default BGK);
    // SimulationFactory.cpp:36-60.
    PP lbm{in, "lbm"};
    std::string lattice = "D3Q19", collision = "BGK";
    if ((rc = lbm.query_str("lattice_type", lattice, found))) return rc;
    if ((rc = lbm.query_str("collision_model", collision, found))) return rc;
    if (lattice == "D2Q9") { d.dim = 2; d.q = 9; }
    else if (lattice == "D3Q15") { d.dim = 3; d.q = 15; }
    else if (lattice == "D3Q19") { d.dim = 3; d.q = 19; }
    else if (lattice == "D3Q27") { d.dim = 3; d.q = 27; }
    else return fail(MPH_ERR_CONFIG, "Unknown or unsupported lbm.lattice_type '" + lattice + "'");
    if (collision == "TRT" || collision == "MRT")
        return fail(MPH_ERR_UNSUPPORTED, "lbm.collision_model '" + collision + "' is a recognised tag but not yet implemented.");
    if (collision != "BGK")
        return fail(MPH_ERR_CONFIG, "Unknown lbm.collision_model '" + collision + "' (expected BGK | TRT | MRT).");
    const int D = d.dim;

    PP grid{in, "grid"}, sim{in, "sim"}, units{in, "units"}, geo{in, "geometry"}, bc{in, "bc"},
        forcing{in, "forcing"}, amr{in, "amr"};

    std::vector<double> nc;
    if ((rc = grid.get_darr("ncells", nc, D))) return rc;
    d.n[0] = d.n[1] = d.n[2] = 1;
    for (int a = 0; a < D; ++a) {
        d.n[a] = (int)nc[a];
        if ((double)d.n[a] != nc[a] || d.n[a] < 1) return fail(MPH_ERR_PARSE, "grid.ncells must be positive integers");
    }
    ri.max_step = 0;
    if (!in.find("sim.max_step")) return fail(MPH_ERR_PARSE, "inputs: missing required key sim.max_step");
    if ((rc = sim.query_int("max_step", ri.max_step, found))) return rc;
    ri.stop_time = -1.0;
    if ((rc = sim.query_double("stop_time", ri.stop_time, found))) return rc;
    ri.plot_int = 100;
    ri.chk_int = 1000;
    if ((rc = amr.query_int("plot_int", ri.plot_int, found))) return rc;
    if ((rc = amr.query_int("chk_int", ri.chk_int, found))) return rc;

    double tau = 0, u_lat = 0, Re = 0, nu_phys = 0;
    bool has_tau = false, has_ulat = false, has_Re = false, has_nu = false;
    if ((rc = lbm.query_double("tau", tau, has_tau))) return rc;
    if ((rc = lbm.query_double("u_lat", u_lat, has_ulat))) return rc;
    if ((rc = units.query_double("Re", Re, has_Re))) return rc;
    if ((rc = units.query_double("nu_phys", nu_phys, has_nu))) return rc;
    double L_ref = 1.0, U_ref = 1.0, rho_ref = 1.0;
    if ((rc = units.query_double("ref_length", L_ref, found))) return rc;
    if ((rc = units.query_double("ref_velocity", U_ref, found))) return rc;
    if ((rc = units.query_double("ref_density", rho_ref, found))) return rc;

    std::vector<double> lo, hi;
    if ((rc = geo.get_darr("prob_lo", lo, D))) return rc;
    if ((rc = geo.get_darr("prob_hi", hi, D))) return rc;
    int use_eb = 0;
    if ((rc = geo.query_int("use_eb", use_eb, found))) return rc;
    if (use_eb != 0)
        return fail(MPH_ERR_UNSUPPORTED, "geometry.use_eb=1: embedded boundaries are not supported");

    // UnitConverter::setGridResolution (Units.cpp:131-167).
    int max_N = d.n[0];
    for (int a = 0; a < D; ++a) max_N = (d.n[a] > max_N) ? d.n[a] : max_N;
    double domLength[3] = {0., 0., 0.}, gridRes[3] = {0., 0., 0.};
    double max_L = -1;
    for (int a = 0; a < D; ++a) {
        domLength[a] = hi[a] - lo[a];
        max_L = (domLength[a] > max_L) ? domLength[a] : max_L;
        gridRes[a] = domLength[a] / double(d.n[a]);
    }
    const double kTol = 1.0e-12;
    if (!(std::abs(gridRes[0] - gridRes[1]) < kTol)) return fail(MPH_ERR_CONFIG, "Lattice must be square (Lx/Nx == Ly/Ny)");
    if (D == 3) {
        if (!(std::abs(gridRes[0] - gridRes[2]) < kTol)) return fail(MPH_ERR_CONFIG, "Lattice must be square (Lx/Nx == Lz/Nz)");
        if (!(std::abs(gridRes[1] - gridRes[2]) < kTol)) return fail(MPH_ERR_CONFIG, "Lattice must be square (Ly/Ny == Lz/Nz)");
    }
    const double dx = max_L / double(max_N);

    // UnitConverter constructor (Units.cpp:20-109).
    if (has_nu) {
        Re = U_ref * L_ref / nu_phys;
        if (has_Re) return fail(MPH_ERR_CONFIG, "UnitConverter: Both units.Re and units.nu_phys were specified.");
    } else if (has_Re) {
        nu_phys = U_ref * L_ref / Re;
    } else {
        return fail(MPH_ERR_CONFIG, "UnitConverter: Neither units.Re nor units.nu_phys were specified.");
    }
    const double cs2 = 1.0 / 3.0;
    double ul;
    if (has_tau) {
        const double nu_lat_from_tau = (tau - 0.5) * cs2;
        const double u_lat_from_tau = nu_lat_from_tau * U_ref * dx / nu_phys;
        if (has_ulat) return fail(MPH_ERR_CONFIG, "UnitConverter: lbm.u_lat and lbm.tau were both specified.");
        ul = u_lat_from_tau;
    } else if (has_ulat) {
        ul = u_lat;
    } else {
        ul = 0.1;
    }
    const double dt = ul * dx / U_ref;
    const double nu_lat = nu_phys * dt / (dx * dx);
    const double tau_d = 0.5 + nu_lat / cs2;
    if (!((tau_d > 0.5) && (tau_d < 2.0)))
        return fail(MPH_ERR_CONFIG, "tau is not within the stability range 0.5 < tau < 2.0 (tau = " + std::to_string(tau_d) + ")");
    if (!(ul < 0.3)) return fail(MPH_ERR_CONFIG, "u_lat does not satisfy the low Mach number limit (u_lat < 0.3)");
    ri.dx = dx; ri.dt = dt; ri.u_lat = ul; ri.nu_lat = nu_lat; ri.tau = tau_d;
    ri.Re = Re; ri.nu_phys = nu_phys; ri.ref_length = L_ref; ri.ref_velocity = U_ref; ri.ref_density = rho_ref;
    d.omega = 1.0 / tau_d;  // SimulationSetup.cpp:54
    ri.omega = d.omega;

    // forcing.accel -> lattice units (SimulationSetup.cpp:56-61).
    std::vector<double> accel;
    if ((rc = forcing.query_darr("accel", accel))) return rc;
    if (!accel.empty() && (int)accel.size() != D)
        return fail(MPH_ERR_CONFIG, "InputParser: forcing.accel must list exactly one component per dimension");
    d.forced = 0;
    for (int a = 0; a < (int)accel.size(); ++a) {
        d.force[a] = accel[a] * dt * dt / dx;  // toLatticeAcceleration, Units.cpp:173
        if (accel[a] != 0.0) d.forced = 1;
    }

    // Boundary names (InputParser.cpp:216-240) and periodicity.
    std::vector<std::string> lon, hin;
    if (!in.find("bc.lo_type") || !in.find("bc.hi_type"))
        return fail(MPH_ERR_PARSE, "inputs: bc.lo_type and bc.hi_type are required");
    bc.query_arr("lo_type", lon);
    bc.query_arr("hi_type", hin);
    if ((int)lon.size() != D || (int)hin.size() != D)
        return fail(MPH_ERR_CONFIG, "bc.lo_type and bc.hi_type must each list exactly one name per direction");
    for (int f = 0; f < 6; ++f) d.face_type[f] = BC_PERIODIC;
    for (int a = 0; a < D; ++a) {
        if ((rc = bc_code(lon[a], d.face_type[2 * a]))) return rc;
        if ((rc = bc_code(hin[a], d.face_type[2 * a + 1]))) return rc;
    }

    // Per-face velocities (InputParser.cpp:22-64, 242-256) and densities
    // (InputParser.cpp:258-268).
    static const char* uw[6] = {"lox_Uwall", "hix_Uwall", "loy_Uwall", "hiy_Uwall", "loz_Uwall", "hiz_Uwall"};
    static const char* ui[6] = {"lox_Uin", "hix_Uin", "loy_Uin", "hiy_Uin", "loz_Uin", "hiz_Uin"};
    static const char* ur[6] = {"lox_rho", "hix_rho", "loy_rho", "hiy_rho", "loz_rho", "hiz_rho"};
    double Uwall[6][3] = {}, Uin[6][3] = {}, frho[6];
    for (int f = 0; f < 2 * D; ++f) {
        std::vector<double> v;
        if ((rc = bc.query_darr(uw[f], v))) return rc;
        if (!v.empty()) {
            if ((int)v.size() != D) return fail(MPH_ERR_CONFIG, std::string("InputParser: bc.") + uw[f] + " must list one component per dimension");
            for (int c = 0; c < D; ++c) {
                if (c == f / 2 && v[c] != 0.)
                    return fail(MPH_ERR_CONFIG, std::string("InputParser: bc.") + uw[f] + " has a nonzero component along the wall normal");
                Uwall[f][c] = v[c];
            }
        }
        if ((rc = bc.query_darr(ui[f], v))) return rc;
        if (!v.empty()) {
            if ((int)v.size() != D) return fail(MPH_ERR_CONFIG, std::string("InputParser: bc.") + ui[f] + " must list one component per dimension");
            for (int c = 0; c < D; ++c) {
                if (c != f / 2 && v[c] != 0.)
                    return fail(MPH_ERR_CONFIG, std::string("InputParser: bc.") + ui[f] + " has a nonzero component tangent to the face");
                Uin[f][c] = v[c];
            }
        }
        frho[f] = rho_ref;
        if ((rc = bc.query_double(ur[f], frho[f], found))) return rc;
        if (!(frho[f] > 0.)) return fail(MPH_ERR_CONFIG, "InputParser: bc.<face>_rho must be positive");
    }
    const double rhoWall = rho_ref / rho_ref;  // toLatticeDensity(refDensity)
    for (int f = 0; f < 2 * D; ++f) {
        const int t = d.face_type[f];
        d.face_rho[f] = 0.0;
        if (t == BC_PERIODIC) continue;
        d.face_rho[f] = rhoWall;
        if (t == BC_MOVING)
            for (int c = 0; c < D; ++c) d.face_U[f][c] = Uwall[f][c] * dt / dx;  // toLatticeVelocity
        else if (t == BC_INFLOW)
            for (int c = 0; c < D; ++c) d.face_U[f][c] = Uin[f][c] * dt / dx;
        else if (t == BC_PRESSURE)
            d.face_rho[f] = frho[f] / rho_ref;
    }
    d.precision = precision;
    mph_resolved_bc table[27];
    if ((rc = resolve_table(d, table))) return rc;
    *desc = d;
    if (info) *info = ri;
    return MPH_OK;
}

}  // extern "C"
