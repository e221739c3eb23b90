// The structure of a block ILU(0) factor (sim/core/math/incomplete_lu.hpp:14-43,
// incomplete_lu.cpp:33-150) prepared for a level-scheduled GPU factorisation and solve.
//
// Each block of rows [block_start[b], block_start[b + 1]) keeps its own couplings (row i:
// the diagonal and its in-block neighbours, sorted by column) and drops the others, so
// the blocks are independent. Inside a block a row depends on the rows of its lower
// columns (factorisation and forward solve) or of its upper columns (backward solve);
// rows of one dependency level run in parallel, the levels in order. The IKJ elimination
// of a row is listed as it runs in the reference: for each lower entry q (column order)
// the pairs (t, at) of value[at] -= value[q] * value[t], so the device factor performs
// the same operations in the same order and gives the same bits.
#pragma once

#include <cstdint>
#include <vector>

namespace psgb {

struct LevelSchedule {
    std::vector<std::uint32_t> block_level;   // [blocks + 1]: each block's levels
    std::vector<std::uint32_t> level_start;   // [levels + 1]: each level's rows in `order`
    std::vector<std::uint32_t> order;         // [rows]
    // The triangular solve's records in `order`'s order, for a solve with the block's x
    // in shared memory: the row and its (at most kIluRecord) couplings of this triangle as
    // block-local indices, and the positions of their values in the factor (packed next
    // to the record after each factorisation). Empty when a block is too large for it.
    std::vector<std::uint16_t> rec_row;       // [rows]
    std::vector<std::uint8_t> rec_count;      // [rows]
    std::vector<std::uint16_t> rec_col;       // [rows][kIluRecord]
    std::vector<std::uint32_t> rec_q;         // [rows][kIluRecord]
    std::uint32_t widest = 0;                 // most rows in one level
};

constexpr int kIluRecord = 8;
constexpr std::uint32_t kIluSharedRows = 4096;   // block rows the shared-memory solve takes

struct IluPattern {
    std::uint32_t rows = 0, blocks = 0;
    std::vector<std::uint32_t> start;      // [rows + 1]
    std::vector<std::uint32_t> column;     // [nnz], sorted per row
    std::vector<std::int32_t> source;      // [nnz]: the CSR entry of the off-diagonal, -1 the diagonal
    std::vector<std::uint32_t> diagonal;   // [rows]: the diagonal's position
    std::vector<std::uint32_t> update_start;   // [nnz + 1]: entry q's updates
    std::vector<std::uint32_t> update_t, update_at;
    LevelSchedule lower, upper;
};

// `offset`/`neighbour`: the matrix's off-diagonal CSR pattern over `rows` rows;
// `block_start`: {0, ..., rows}. Throws std::invalid_argument if they do not match.
IluPattern ilu_pattern(const std::vector<std::uint32_t>& offset, const std::vector<std::uint32_t>& neighbour,
                       const std::vector<std::uint32_t>& block_start);

// {0, 256, 512, ..., rows}: the reference's fixed 256-row blocks, scaled by `stride`
// rows per node (the tracer's stacked layers).
std::vector<std::uint32_t> fixed_blocks(std::uint32_t nodes, std::uint32_t stride);

}  // namespace psgb
