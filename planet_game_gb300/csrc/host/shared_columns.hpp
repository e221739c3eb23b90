// The fine level's ELL columns once per distinct graph of a batch (host side).
//
// Planets of one mesh level have the same graph whatever their radius. A batch holding two
// or more of them keeps their planet-local columns once per distinct graph; a tile finds
// its planet's copy through a shift: column j of batch row r is
//   shift[0] + scol[j * pitch + (r - shift[1])]
// where shift[0] is the planet's first row in the batch and shift[1] that row minus its
// graph's first row in scol. A missing neighbour slot and every padding row point at the
// row itself, as in the per-planet columns.
#pragma once

#include "hierarchy.hpp"

#include <cstddef>
#include <cstdint>
#include <vector>

namespace psgb {

struct SharedColumns {
    std::uint32_t pitch = 0;            // rows of the distinct graphs, each padded to whole tiles; 0: none shared
    std::vector<std::int32_t> scol;     // [width][pitch] planet-local columns
    std::vector<std::int32_t> shift;    // [tiles][2] per tile: planet's first row, that row minus its graph's first row
};

// `fine[i]`: planet i's fine level (size, CSR offset and column); `base[i]`: its first row
// in the batch (every planet padded to whole 256-row tiles); `tile_inst[t]`: the planet of
// tile t. Returns pitch 0 when no two planets share a graph.
SharedColumns shared_columns(const std::vector<const HostLevel*>& fine, const std::vector<std::int64_t>& base,
                             const std::vector<std::int32_t>& tile_inst, std::size_t width);

}  // namespace psgb
