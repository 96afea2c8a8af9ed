// mph_internal.h -- declarations shared by the host translation units of
// libmph (configuration, simulation handle, kernels).
#pragma once

#include "mph.h"

#include <string>
#include <utility>
#include <vector>

namespace mph {

// Records the calling thread's last error message; returns `code`.
int fail(int code, const std::string& msg);
void clear_error();

// One definition of an inputs file: key and its value tokens.
struct Def {
    std::string key;
    std::vector<std::string> vals;
};

// Parsed inputs (ParmParse subset): definitions in order; the last
// definition of a key wins (ParmParse's default "last" query).
struct Inputs {
    std::vector<Def> defs;
    const Def* find(const std::string& key) const;
};

// Validates `d` and fills the 27-entry resolved table (BCManager::finalize).
// Returns MPH_OK or an error code (message recorded).
int resolve_table(const mph_desc& d, mph_resolved_bc* table);

// Lattice (dim, q) validity.
bool lattice_ok(int dim, int q);

}  // namespace mph
