// Agglomeration of a mesh onto the mesh one level coarser (see agglomerate.hpp), restating
// build_agglomeration (sim/planet/surface/heat_transport.cpp:467-512): integer groups and
// summed areas bit-identical to the reference's.
#include "agglomerate.hpp"

#include <stdexcept>

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

Agglomeration agglomerate(const HostMesh& fine, const HostMesh& coarse) {
    Agglomeration out;
    out.group_of_cell.resize(fine.cells);
    out.area_m2.assign(coarse.cells, 0.0);
    std::size_t guess = 0;
    for (std::size_t cell = 0; cell < fine.cells; ++cell) {
        const double* centre = &fine.center[3 * cell];
        for (;;) {
            std::size_t best = guess;
            double best_dot = dot3(centre, &coarse.center[3 * guess]);
            const std::uint32_t begin = coarse.edge_offset[guess];
            for (std::uint32_t k = 0; k < coarse.edge_count[guess]; ++k) {
                const std::size_t other = coarse.nb_cell[begin + k];
                const double value = dot3(centre, &coarse.center[3 * other]);
                if (value > best_dot) {
                    best_dot = value;
                    best = other;
                }
            }
            if (best == guess) break;
            guess = best;
        }
        out.group_of_cell[cell] = static_cast<std::uint32_t>(guess);
        out.area_m2[guess] += fine.area_m2[cell];
    }
    for (double area : out.area_m2) {
        if (!(area > 0.0)) throw std::logic_error("a coarse transport cell received no fine cell");
    }
    out.fine_area_m2 = fine.area_m2;
    list_members(out, coarse.cells);
    return out;
}

}  // namespace psgb
