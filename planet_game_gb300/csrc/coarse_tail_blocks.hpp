// The spread coarse tail's layout of blocks per planet (host arithmetic, host/tail_blocks.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace psgb {

// Blocks per planet for a tail from some level: `rows[i]` planet i's rows there, `budget`
// blocks that can be co-resident; each planet gets at least one, the rest go one at a
// time to the planet with the most rows per block (at most 16 each, while a block would
// cover more than 2048 rows). Returns the packed per-block words: planet | rank << 16 |
// blocks << 24.
std::vector<std::uint32_t> tail_blocks(const std::vector<std::uint32_t>& rows, unsigned budget);

}  // namespace psgb
