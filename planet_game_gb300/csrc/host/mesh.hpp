// Host-side planet mesh and transport graph, structure-of-arrays.
//
// HostMesh holds what the reference PlanetMesh holds (sim/planet/mesh/planet_mesh.hpp:44-125),
// laid out as flat arrays so that it can be uploaded to HBM and handed through the
// C-ABI without C++ types. TransportGraph mirrors the reference's CSR transport
// graph (sim/planet/surface/heat_transport.hpp:27-36).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace psgb {

// Fixed 256-cell blocks, as the reference's deterministic blocks
// (planet_mesh.hpp:76): reductions sum per block, then over blocks in order.
inline constexpr std::size_t cell_block = 256;

struct HostMesh {
    std::uint32_t level = 0;
    double radius_m = 0.0;
    std::size_t cells = 0, edges = 0, corners = 0, directed = 0;

    // per cell
    std::vector<double> center, east, north;   // 3 per cell
    std::vector<double> area_m2;
    std::vector<std::uint32_t> source_vertex, edge_offset;
    std::vector<std::uint8_t> edge_count;
    // per directed edge (CSR by cell, counter-clockwise from the reference's atan2 order)
    std::vector<std::uint32_t> nb_cell, nb_edge, nb_corner;
    std::vector<float> normal_east, normal_north;
    // per undirected edge
    std::vector<std::uint32_t> edge_first, edge_second;
    std::vector<double> edge_length_m, edge_distance_m;
    // per corner (dual vertex = primal face circumcentre)
    std::vector<double> corner_unit;            // 3 per corner
};

HostMesh build_icosphere(std::uint32_t level, double radius_m);

std::size_t icosphere_cell_count(std::uint32_t level);

struct TransportGraph {
    std::vector<double> area_m2;
    std::vector<std::uint32_t> offset;      // cells + 1
    std::vector<std::uint32_t> neighbour;
    std::vector<double> weight;             // l / d
    std::vector<double> weight_sum;
    std::size_t size() const { return area_m2.size(); }
};

TransportGraph transport_graph(const HostMesh& mesh);

}  // namespace psgb
