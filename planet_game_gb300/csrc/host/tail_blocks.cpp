// Blocks per planet for the spread coarse tail (see coarse_tail.hpp): host arithmetic only.
#include "../coarse_tail_blocks.hpp"

#include <stdexcept>

namespace psgb {

std::vector<std::uint32_t> tail_blocks(const std::vector<std::uint32_t>& rows, unsigned budget) {
    const std::size_t I = rows.size();
    std::vector<unsigned> size(I, 1);
    if (I > 0xFFFFu) throw std::logic_error("coarse tail: too many planets for per-planet blocks");
    unsigned used = static_cast<unsigned>(I);
    while (used < budget) {
        std::size_t best = I;
        double most = 0.0;
        for (std::size_t i = 0; i < I; ++i) {
            const double per = static_cast<double>(rows[i]) / size[i];
            if (size[i] < 16 && per > most) { most = per; best = i; }
        }
        if (best == I || most <= 2048.0) break;   // a block covers up to 2048 rows well
        ++size[best];
        ++used;
    }
    std::vector<std::uint32_t> cta;
    for (std::size_t i = 0; i < I; ++i)
        for (unsigned r = 0; r < size[i]; ++r) cta.push_back(static_cast<std::uint32_t>(i) | (r << 16) | (size[i] << 24));
    return cta;
}

}  // namespace psgb
