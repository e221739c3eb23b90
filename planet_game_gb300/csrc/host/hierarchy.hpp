// Aggregation-multigrid hierarchy structure, built on the host.
//
// The structure (aggregates, coarse sparsity patterns, the Galerkin scatter
// targets and the level count) is integer data and must equal the reference's
// bit for bit: aggregate_rows, coarsen_pattern, coarsen_values and
// build_hierarchy in sim/planet/surface/heat_transport.cpp:73-200. The values
// used to choose aggregates on the coarse levels are the unit-conductance
// Galerkin values, summed in the reference's order.
//
// Only the structure lives here. The device holds the values (ELL, slot-major)
// and recomputes the Galerkin values whenever the matrix changes, from the
// gather lists built below, in the reference's summation order.
#pragma once

#include "mesh.hpp"

#include <cstdint>
#include <vector>

namespace psgb {

inline constexpr std::uint32_t coarsest_rows = 400;   // heat_transport.cpp:188

struct HostLevel {
    std::uint32_t size = 0;
    // CSR off-diagonal pattern (fine level: the transport graph's order).
    std::vector<std::uint32_t> offset, column;
    std::vector<double> diagonal, value;            // unit-conductance values
    std::vector<std::uint32_t> aggregate;           // empty on the coarsest level
    std::vector<std::int64_t> target;               // -1: the aggregate's diagonal
    std::uint32_t width = 0;                        // max off-diagonals per row
};

struct HostHierarchy {
    std::vector<HostLevel> levels;
};

HostHierarchy build_hierarchy(const TransportGraph& graph);

inline std::uint32_t pad_rows(std::uint32_t n) { return (n + 255u) / 256u * 256u; }

// ELL width used on the device for a level whose rows have at most `w`
// off-diagonals: the kernels are specialised for 6, 8, 12 and 16.
std::uint32_t device_width(std::uint32_t w);

}  // namespace psgb
