// The agglomerated transport graph: the transport one mesh level coarser, as the
// reference's production path runs it (sim/planet/surface/heat_transport.cpp:456-543,
// agglomerated_transport_graph / agglomerated_mesh).
#pragma once

#include "mesh.hpp"

#include <cstdint>
#include <vector>

namespace psgb {

struct Agglomeration {
    std::vector<std::uint32_t> group_of_cell;   // fine cell -> group (a cell of the coarser mesh)
    std::vector<double> area_m2;                // per group: the sum of its fine cells' areas
    std::vector<std::uint32_t> member_offset;   // [groups + 1]: each group's fine cells ...
    std::vector<std::uint32_t> member;          // ... in cell order
    std::vector<double> fine_area_m2;           // the fine cells' own areas
};

// The identity grouping of a mesh onto itself (level 0).
Agglomeration identity_agglomeration(const HostMesh& mesh);

// Each fine cell joins the nearest cell of `coarse` (the mesh one level coarser), found by
// a greedy walk over the coarse mesh that starts from the previous fine cell's answer;
// group areas sum the fine areas in fine-cell order. Throws std::logic_error if a group
// receives no cell.
Agglomeration agglomerate(const HostMesh& fine, const HostMesh& coarse);

}  // namespace psgb
