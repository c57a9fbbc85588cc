// mg_internal.h -- shared internals of libmg (host side; no device code here).
#pragma once

#include "mg.h"

#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

struct mg_host_graph {
    int32_t nv = 0, ne = 0, start_p = 0, tra = 0;
    std::vector<int32_t> v, e, ev;  // CSR row offsets, column ids, integer weights
    bool pinned = false;
    // page-locked copies of v / e / ev made by mg_host_graph_pin (driver
    // allocations: staged uploads read them at full link speed)
    int32_t *pin_v = nullptr, *pin_e = nullptr, *pin_ev = nullptr;
};

namespace mgi {

// Thread-local error message; fail() records it and returns the status.
mg_status fail(mg_status s, const char *fmt, ...);
void clear_error();

// Number of host threads for a request of n (0 or less = all online cores).
int host_threads(int n);

// Allocation failure injection for tests: MG_FAIL_ALLOC_AT=k makes the k-th
// counted allocation (host or device, 1-based, process-wide) fail.
bool inject_alloc_failure();

// Loader pipeline shared by mg_load_mtx, mg_host_graph_from_entries and the
// generators: expands symmetric entries, sorts by (src, dst, file order),
// drops duplicates (and src >= dst edges under CC), removes unused vertices,
// renumbers the source and builds the CSR -- read_input.cu:88-171.
struct Entries {
    int32_t nv_decl = 0;
    std::vector<int32_t> src, dst, val;  // val empty -> pattern weights from seed
};
mg_status build_csr(const Entries &in, bool sym, bool cc, int32_t source, uint64_t seed, int nthreads,
                    mg_host_graph *out);

uint32_t pattern_weight(uint64_t seed, uint64_t entry);

}  // namespace mgi
