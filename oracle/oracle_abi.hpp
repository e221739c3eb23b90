// CPU ORACLE - test infrastructure only. The flat graph both oracle files take from the
// tests (the product's host builder's arrays, pinned to the reference's).
#pragma once

#include <cstdint>

extern "C" {

struct orc_graph {
    std::uint64_t n;
    const std::uint32_t* offset;      // n + 1
    const std::uint32_t* neighbour;
    const double* weight;             // l / d
    const double* weight_sum;
    const double* area;
};

// planetsim_oracle.cpp: the aggregation hierarchy with its SGS V-cycle (GraphMultigrid).
void* orc_hierarchy_new(const orc_graph* g);
void orc_hierarchy_free(void* h);
void orc_hierarchy_set_matrix(void* h, const double* diag, const double* off);
void orc_vcycle_sgs(void* h, const double* rhs, double* out);
}
