// Agglomeration of a mesh onto the mesh one level coarser (see agglomerate.hpp), restating
// build_agglomeration (sim/planet/surface/heat_transport.cpp:467-512): integer groups and
// summed areas bit-identical to the reference's.
#include "agglomerate.hpp"

#include <stdexcept>
#include <string>

namespace psgb {

namespace {

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Each group's fine cells in cell order (a counting sort; surface_energy.cpp:1225-1238
// lists the members the same way for its group means).
void list_members(Agglomeration& a, std::size_t groups) {
    a.member_offset.assign(groups + 1, 0);
    for (std::uint32_t g : a.group_of_cell) ++a.member_offset[g + 1];
    for (std::size_t g = 0; g < groups; ++g) a.member_offset[g + 1] += a.member_offset[g];
    a.member.resize(a.group_of_cell.size());
    std::vector<std::uint32_t> next(a.member_offset.begin(), a.member_offset.end() - 1);
    for (std::size_t c = 0; c < a.group_of_cell.size(); ++c) a.member[next[a.group_of_cell[c]]++] = static_cast<std::uint32_t>(c);
}

}  // namespace

Agglomeration identity_agglomeration(const HostMesh& mesh) {
    Agglomeration out;
    out.group_of_cell.resize(mesh.cells);
    for (std::size_t c = 0; c < mesh.cells; ++c) out.group_of_cell[c] = static_cast<std::uint32_t>(c);
    out.area_m2 = mesh.area_m2;
    out.fine_area_m2 = mesh.area_m2;
    list_members(out, mesh.cells);
    return out;
}

// The coarse node nearest to `point` (largest dot product of unit centres), found by
// descending from `start`: move to the best of the current node's neighbours while one
// beats it strictly, the first of equals winning. Consecutive fine cells lie close
// together, so starting at the previous cell's node makes the descent short; the start
// and the strict test decide between equidistant nodes exactly as the reference's walk
// (heat_transport.cpp:483-500) does.
std::size_t descend_to_nearest(const HostMesh& coarse, std::size_t start, const double* point) {
    std::size_t at = start;
    for (;;) {
        const double here = dot3(point, &coarse.center[3 * at]);
        double better = here;
        std::size_t next = at;
        const std::uint32_t* ring = &coarse.nb_cell[coarse.edge_offset[at]];
        for (std::uint32_t k = 0; k < coarse.edge_count[at]; ++k) {
            const double d = dot3(point, &coarse.center[3 * ring[k]]);
            if (d > better) {
                better = d;
                next = ring[k];
            }
        }
        if (next == at) return at;
        at = next;
    }
}

Agglomeration agglomerate(const HostMesh& fine, const HostMesh& coarse) {
    Agglomeration out;
    out.group_of_cell.resize(fine.cells);
    out.area_m2.assign(coarse.cells, 0.0);
    std::size_t node = 0;
    for (std::size_t cell = 0; cell < fine.cells; ++cell) {
        node = descend_to_nearest(coarse, node, &fine.center[3 * cell]);
        out.group_of_cell[cell] = static_cast<std::uint32_t>(node);
        out.area_m2[node] += fine.area_m2[cell];
    }
    for (std::size_t g = 0; g < coarse.cells; ++g) {
        if (!(out.area_m2[g] > 0.0)) {
            throw std::logic_error("agglomeration: coarse node " + std::to_string(g) + " of " +
                                   std::to_string(coarse.cells) + " gathered no fine cell");
        }
    }
    out.fine_area_m2 = fine.area_m2;
    list_members(out, coarse.cells);
    return out;
}

}  // namespace psgb
