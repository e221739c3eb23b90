// Host-side aggregation hierarchy: structure bit-identical to the reference's
// build_hierarchy (sim/planet/surface/heat_transport.cpp:73-200).
//
// aggregate_rows (:73-108): greedy pass in row order - a free row whose
// neighbours are all free seeds an aggregate with them; leftovers join their
// strongest (most negative off-diagonal) aggregated neighbour, else form their own.
// coarsen_pattern (:113-154): coarse columns sorted and unique per coarse row;
// every fine off-diagonal lands on a coarse off-diagonal or the diagonal.
// coarsen_values (:157-171): values summed in fine-row order.
#include "hierarchy.hpp"

#include <algorithm>
#include <limits>
#include <stdexcept>

namespace psgb {
namespace {

constexpr std::uint32_t unassigned = std::numeric_limits<std::uint32_t>::max();

std::vector<std::uint32_t> aggregate_rows(const HostLevel& level, std::uint32_t& count) {
    std::vector<std::uint32_t> agg(level.size, unassigned);
    count = 0;
    for (std::uint32_t row = 0; row < level.size; ++row) {
        bool free = agg[row] == unassigned;
        for (std::uint32_t k = level.offset[row]; free && k < level.offset[row + 1]; ++k) {
            free = agg[level.column[k]] == unassigned;
        }
        if (!free) continue;
        agg[row] = count;
        for (std::uint32_t k = level.offset[row]; k < level.offset[row + 1]; ++k) {
            agg[level.column[k]] = count;
        }
        ++count;
    }
    for (std::uint32_t row = 0; row < level.size; ++row) {
        if (agg[row] != unassigned) continue;
        double strongest = 0.0;
        for (std::uint32_t k = level.offset[row]; k < level.offset[row + 1]; ++k) {
            const std::uint32_t other = level.column[k];
            if (agg[other] != unassigned && -level.value[k] > strongest) {
                strongest = -level.value[k];
                agg[row] = agg[other];
            }
        }
        if (agg[row] == unassigned) agg[row] = count++;
    }
    return agg;
}

HostLevel coarsen_pattern(HostLevel& fine) {
    std::uint32_t count = 0;
    fine.aggregate = aggregate_rows(fine, count);
    HostLevel coarse;
    coarse.size = count;
    std::vector<std::vector<std::uint32_t>> columns(count);
    for (std::uint32_t row = 0; row < fine.size; ++row) {
        const std::uint32_t a = fine.aggregate[row];
        for (std::uint32_t k = fine.offset[row]; k < fine.offset[row + 1]; ++k) {
            const std::uint32_t b = fine.aggregate[fine.column[k]];
            if (b != a) columns[a].push_back(b);
        }
    }
    coarse.offset.assign(count + 1, 0);
    for (std::uint32_t row = 0; row < count; ++row) {
        auto& entries = columns[row];
        std::sort(entries.begin(), entries.end());
        entries.erase(std::unique(entries.begin(), entries.end()), entries.end());
        coarse.column.insert(coarse.column.end(), entries.begin(), entries.end());
        coarse.offset[row + 1] = static_cast<std::uint32_t>(coarse.column.size());
        coarse.width = std::max<std::uint32_t>(coarse.width, static_cast<std::uint32_t>(entries.size()));
    }
    coarse.diagonal.assign(count, 0.0);
    coarse.value.assign(coarse.column.size(), 0.0);
    fine.target.assign(fine.column.size(), -1);
    for (std::uint32_t row = 0; row < fine.size; ++row) {
        const std::uint32_t a = fine.aggregate[row];
        for (std::uint32_t k = fine.offset[row]; k < fine.offset[row + 1]; ++k) {
            const std::uint32_t b = fine.aggregate[fine.column[k]];
            if (b == a) continue;
            const auto first = coarse.column.begin() + coarse.offset[a];
            const auto last = coarse.column.begin() + coarse.offset[a + 1];
            fine.target[k] = std::lower_bound(first, last, b) - coarse.column.begin();
        }
    }
    return coarse;
}

void coarsen_values(const HostLevel& fine, HostLevel& coarse) {
    std::fill(coarse.diagonal.begin(), coarse.diagonal.end(), 0.0);
    std::fill(coarse.value.begin(), coarse.value.end(), 0.0);
    for (std::uint32_t row = 0; row < fine.size; ++row) {
        const std::uint32_t a = fine.aggregate[row];
        coarse.diagonal[a] += fine.diagonal[row];
        for (std::uint32_t k = fine.offset[row]; k < fine.offset[row + 1]; ++k) {
            if (fine.target[k] < 0) {
                coarse.diagonal[a] += fine.value[k];
            } else {
                coarse.value[static_cast<std::size_t>(fine.target[k])] += fine.value[k];
            }
        }
    }
}

}  // namespace

HostHierarchy build_hierarchy(const TransportGraph& graph) {
    HostHierarchy h;
    h.levels.resize(1);
    HostLevel& fine = h.levels.front();
    fine.size = static_cast<std::uint32_t>(graph.size());
    fine.diagonal = graph.weight_sum;
    fine.offset = graph.offset;
    fine.column = graph.neighbour;
    fine.value.resize(graph.weight.size());
    for (std::size_t k = 0; k < graph.weight.size(); ++k) fine.value[k] = -graph.weight[k];
    for (std::uint32_t r = 0; r < fine.size; ++r) {
        fine.width = std::max(fine.width, fine.offset[r + 1] - fine.offset[r]);
    }
    while (h.levels.back().size > coarsest_rows) {
        HostLevel coarse = coarsen_pattern(h.levels.back());
        coarsen_values(h.levels.back(), coarse);
        if (coarse.size >= h.levels.back().size) {
            h.levels.back().aggregate.clear();
            h.levels.back().target.clear();
            break;
        }
        h.levels.push_back(std::move(coarse));
    }
    return h;
}

std::uint32_t device_width(std::uint32_t w) {
    if (w <= 6) return 6;
    if (w <= 8) return 8;
    if (w <= 12) return 12;
    if (w <= 16) return 16;
    throw std::logic_error("multigrid level wider than 16 off-diagonals per row");
}

}  // namespace psgb
