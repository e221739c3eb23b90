// Host check of the spread coarse tail's block layout (planet_game_gb300/csrc/host/
// tail_blocks.cpp), run by tests/test_ilu_pattern_host.py: every planet gets its blocks
// contiguously with ranks 0..size-1, at least one and at most 16, the total within the
// budget, extra blocks going to the planets with the most rows per block.
#include "coarse_tail_blocks.hpp"

#include <cstdio>
#include <vector>

using namespace psgb;

static int fail(const char* what) {
    std::printf("FAIL %s\n", what);
    return 1;
}

int main() {
    // the 64-planet mix at level 1: 16 x 162, 24 x 642, 16 x 2562, 8 x 10242 rows
    std::vector<std::uint32_t> rows;
    for (int i = 0; i < 16; ++i) rows.push_back(162);
    for (int i = 0; i < 24; ++i) rows.push_back(642);
    for (int i = 0; i < 16; ++i) rows.push_back(2562);
    for (int i = 0; i < 8; ++i) rows.push_back(10242);
    for (unsigned budget : {64u, 100u, 152u, 1000u}) {
        const std::vector<std::uint32_t> cta = tail_blocks(rows, budget);
        if (cta.size() > std::max<std::size_t>(budget, rows.size())) return fail("over budget");
        std::vector<unsigned> count(rows.size(), 0), size(rows.size(), 0);
        std::uint32_t previous = 0;
        for (std::size_t k = 0; k < cta.size(); ++k) {
            const std::uint32_t planet = cta[k] & 0xFFFFu, rank = (cta[k] >> 16) & 0xFFu, sz = cta[k] >> 24;
            if (planet < previous) return fail("planets out of order");
            previous = planet;
            if (rank != count[planet]) return fail("ranks not 0..size-1 in order");
            ++count[planet];
            size[planet] = sz;
        }
        for (std::size_t i = 0; i < rows.size(); ++i) {
            if (count[i] != size[i] || size[i] < 1 || size[i] > 16) return fail("block count");
            if (rows[i] <= 2048 && size[i] != 1) return fail("a small planet took extra blocks");
        }
        if (budget >= 152 && size.back() < 5) return fail("the largest planets did not spread");
    }
    if (tail_blocks(rows, 10).size() != rows.size()) return fail("a budget below one block each");
    std::printf("OK\n");
    return 0;
}
