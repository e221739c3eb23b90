// Block ILU(0) structure and level schedules (see ilu_pattern.hpp).
#include "ilu_pattern.hpp"

#include <algorithm>
#include <limits>
#include <stdexcept>
#include <utility>

namespace psgb {

namespace {

// Rows of each block grouped by dependency level: level(i) = 1 + max level of the rows
// it depends on (`depends(i, f)` calls f(j) for each), rows visited in `forward` order.
template <typename Depends>
LevelSchedule schedule(const std::vector<std::uint32_t>& block_start, bool forward, Depends&& depends) {
    LevelSchedule s;
    const std::uint32_t rows = block_start.back();
    std::vector<std::uint32_t> level(rows, 0);
    s.block_level.push_back(0);
    s.level_start.push_back(0);
    for (std::size_t b = 0; b + 1 < block_start.size(); ++b) {
        const std::uint32_t first = block_start[b], last = block_start[b + 1];
        std::uint32_t depth = 0;
        for (std::uint32_t n = 0; n < last - first; ++n) {
            const std::uint32_t i = forward ? first + n : last - 1 - n;
            std::uint32_t l = 0;
            depends(i, [&](std::uint32_t j) { l = std::max(l, level[j] + 1); });
            level[i] = l;
            depth = std::max(depth, l + 1);
        }
        std::vector<std::vector<std::uint32_t>> by_level(depth);
        for (std::uint32_t i = first; i < last; ++i) by_level[level[i]].push_back(i);
        for (const auto& rows_of_level : by_level) {
            s.order.insert(s.order.end(), rows_of_level.begin(), rows_of_level.end());
            s.level_start.push_back(static_cast<std::uint32_t>(s.order.size()));
        }
        s.block_level.push_back(static_cast<std::uint32_t>(s.level_start.size() - 1));
    }
    return s;
}

}  // namespace

std::vector<std::uint32_t> fixed_blocks(std::uint32_t nodes, std::uint32_t stride) {
    std::vector<std::uint32_t> out{0};
    for (std::uint32_t begin = 0; begin < nodes; begin += 256) out.push_back(std::min(nodes, begin + 256) * stride);
    return out;
}

IluPattern ilu_pattern(const std::vector<std::uint32_t>& offset, const std::vector<std::uint32_t>& neighbour,
                       const std::vector<std::uint32_t>& block_start) {
    if (offset.empty() || offset.back() != neighbour.size() || block_start.size() < 2 || block_start.front() != 0 ||
        block_start.back() != offset.size() - 1) {
        throw std::invalid_argument("incomplete LU: the pattern does not match");
    }
    for (std::size_t b = 0; b + 1 < block_start.size(); ++b) {
        if (block_start[b + 1] < block_start[b]) throw std::invalid_argument("incomplete LU: the pattern does not match");
    }
    IluPattern p;
    p.rows = static_cast<std::uint32_t>(offset.size() - 1);
    p.blocks = static_cast<std::uint32_t>(block_start.size() - 1);
    std::vector<std::uint32_t> block_of(p.rows);
    for (std::uint32_t b = 0; b < p.blocks; ++b)
        for (std::uint32_t i = block_start[b]; i < block_start[b + 1]; ++i) block_of[i] = b;
    for (std::uint32_t k = 0; k < neighbour.size(); ++k) {
        if (neighbour[k] >= p.rows) throw std::invalid_argument("incomplete LU: the pattern does not match");
    }
    // Rows: the diagonal and the in-block couplings, sorted by column (a stable sort
    // keeps the CSR order of repeated columns, as the reference's std::sort need not;
    // the transport patterns have none).
    p.start.assign(p.rows + 1, 0);
    p.diagonal.resize(p.rows);
    std::vector<std::pair<std::uint32_t, std::int32_t>> row;
    for (std::uint32_t i = 0; i < p.rows; ++i) {
        row.clear();
        row.emplace_back(i, -1);
        for (std::uint32_t k = offset[i]; k < offset[i + 1]; ++k)
            if (block_of[neighbour[k]] == block_of[i]) row.emplace_back(neighbour[k], static_cast<std::int32_t>(k));
        std::stable_sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (const auto& [c, k] : row) {
            if (c == i) p.diagonal[i] = static_cast<std::uint32_t>(p.column.size());
            p.column.push_back(c);
            p.source.push_back(k);
        }
        p.start[i + 1] = static_cast<std::uint32_t>(p.column.size());
    }
    // The IKJ elimination's updates (incomplete_lu.cpp:108-135), in its loop order.
    const std::uint32_t absent = std::numeric_limits<std::uint32_t>::max();
    std::vector<std::uint32_t> position(p.rows, absent);
    p.update_start.assign(p.column.size() + 1, 0);
    for (std::uint32_t i = 0; i < p.rows; ++i) {
        for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q) position[p.column[q]] = q;
        for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q) {
            if (q < p.diagonal[i]) {
                const std::uint32_t j = p.column[q];
                for (std::uint32_t t = p.diagonal[j] + 1; t < p.start[j + 1]; ++t) {
                    const std::uint32_t at = position[p.column[t]];
                    if (at != absent) {
                        p.update_t.push_back(t);
                        p.update_at.push_back(at);
                    }
                }
            }
            p.update_start[q + 1] = static_cast<std::uint32_t>(p.update_t.size());
        }
        for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q) position[p.column[q]] = absent;
    }
    p.lower = schedule(block_start, true, [&](std::uint32_t i, auto&& f) {
        for (std::uint32_t q = p.start[i]; q < p.diagonal[i]; ++q) f(p.column[q]);
    });
    p.upper = schedule(block_start, false, [&](std::uint32_t i, auto&& f) {
        for (std::uint32_t q = p.diagonal[i] + 1; q < p.start[i + 1]; ++q) f(p.column[q]);
    });
    // Records for the shared-memory solve, if every block and row fit it.
    bool fits = true;
    for (std::uint32_t b = 0; b < p.blocks; ++b)
        fits = fits && block_start[b + 1] - block_start[b] <= kIluSharedRows;
    for (std::uint32_t i = 0; i < p.rows && fits; ++i)
        fits = p.diagonal[i] - p.start[i] <= static_cast<std::uint32_t>(kIluRecord) &&
               p.start[i + 1] - p.diagonal[i] - 1 <= static_cast<std::uint32_t>(kIluRecord);
    if (fits) {
        for (int part = 0; part < 2; ++part) {
            LevelSchedule& s = part == 0 ? p.lower : p.upper;
            s.rec_row.resize(p.rows);
            s.rec_count.resize(p.rows);
            s.rec_col.assign(std::size_t(p.rows) * kIluRecord, 0);
            s.rec_q.assign(std::size_t(p.rows) * kIluRecord, 0);
            for (std::uint32_t b = 0; b < p.blocks; ++b) {
                for (std::uint32_t lv = s.block_level[b]; lv < s.block_level[b + 1]; ++lv) {
                    s.widest = std::max(s.widest, s.level_start[lv + 1] - s.level_start[lv]);
                    for (std::uint32_t idx = s.level_start[lv]; idx < s.level_start[lv + 1]; ++idx) {
                        const std::uint32_t i = s.order[idx];
                        const std::uint32_t first = block_start[b];
                        const std::uint32_t q0 = part == 0 ? p.start[i] : p.diagonal[i] + 1;
                        const std::uint32_t q1 = part == 0 ? p.diagonal[i] : p.start[i + 1];
                        s.rec_row[idx] = static_cast<std::uint16_t>(i - first);
                        s.rec_count[idx] = static_cast<std::uint8_t>(q1 - q0);
                        for (std::uint32_t q = q0; q < q1; ++q) {
                            s.rec_col[std::size_t(idx) * kIluRecord + (q - q0)] = static_cast<std::uint16_t>(p.column[q] - first);
                            s.rec_q[std::size_t(idx) * kIluRecord + (q - q0)] = q;
                        }
                    }
                }
            }
        }
    }
    return p;
}

}  // namespace psgb
