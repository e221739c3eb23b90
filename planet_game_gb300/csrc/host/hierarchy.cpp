// Host-side aggregation hierarchy. Its integer structure must equal the one the
// reference's build_hierarchy produces (sim/planet/surface/heat_transport.cpp:73-200),
// so the rules below are the reference's; the code is organised around claims,
// coupling pairs and per-aggregate member lists instead.
//
// Aggregation rule (:73-108): walking rows in order, a row whose whole neighbourhood is
// still unclaimed claims it as a new aggregate. Rows left over are then visited in order;
// each joins the aggregate of the neighbour it is most strongly coupled to (largest
// -a_ij, strictly above zero, the first such neighbour on ties, claims made earlier in
// this second walk included), or opens an aggregate of its own.
// Coarse pattern (:113-154): the coarse row of an aggregate couples to every other
// aggregate one of its members touches, columns in ascending order; each fine
// off-diagonal lands on one coarse off-diagonal, or on the coarse diagonal when both ends
// share an aggregate. Galerkin values (:157-171): summed in fine-row order.
#include "hierarchy.hpp"

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <utility>

namespace psgb {
namespace {

constexpr std::int64_t kUnclaimed = -1;

// Aggregate of every row of `level`; `aggregates` receives their number.
std::vector<std::uint32_t> claim_aggregates(const HostLevel& level, std::uint32_t& aggregates) {
    std::vector<std::int64_t> owner(level.size, kUnclaimed);
    std::int64_t opened = 0;
    const auto neighbours = [&](std::uint32_t row) {
        return std::make_pair(level.column.begin() + level.offset[row], level.column.begin() + level.offset[row + 1]);
    };
    // first walk: seeds with their whole neighbourhood
    for (std::uint32_t row = 0; row < level.size; ++row) {
        const auto [first, last] = neighbours(row);
        const bool untouched = owner[row] == kUnclaimed &&
                               std::all_of(first, last, [&](std::uint32_t c) { return owner[c] == kUnclaimed; });
        if (!untouched) continue;
        owner[row] = opened;
        std::for_each(first, last, [&](std::uint32_t c) { owner[c] = opened; });
        ++opened;
    }
    // second walk: leftovers follow their strongest claimed coupling
    for (std::uint32_t row = 0; row < level.size; ++row) {
        if (owner[row] != kUnclaimed) continue;
        double pull = 0.0;
        std::int64_t chosen = kUnclaimed;
        for (std::uint32_t k = level.offset[row]; k < level.offset[row + 1]; ++k) {
            const std::int64_t there = owner[level.column[k]];
            const double coupling = -level.value[k];
            if (there == kUnclaimed || !(coupling > pull)) continue;
            pull = coupling;
            chosen = there;
        }
        owner[row] = chosen != kUnclaimed ? chosen : opened++;
    }
    aggregates = static_cast<std::uint32_t>(opened);
    return std::vector<std::uint32_t>(owner.begin(), owner.end());
}

// Fine rows of each aggregate, ascending: offsets [aggregates + 1] and rows.
void members_of(const std::vector<std::uint32_t>& aggregate, std::uint32_t aggregates,
                std::vector<std::uint32_t>& start, std::vector<std::uint32_t>& rows) {
    start.assign(aggregates + 1, 0);
    for (std::uint32_t a : aggregate) ++start[a + 1];
    for (std::uint32_t a = 0; a < aggregates; ++a) start[a + 1] += start[a];
    rows.resize(aggregate.size());
    std::vector<std::uint32_t> fill(start.begin(), start.end() - 1);
    for (std::uint32_t r = 0; r < aggregate.size(); ++r) rows[fill[aggregate[r]]++] = r;
}

HostLevel coarsen_pattern(HostLevel& fine) {
    std::uint32_t aggregates = 0;
    fine.aggregate = claim_aggregates(fine, aggregates);
    const std::vector<std::uint32_t>& agg = fine.aggregate;
    HostLevel coarse;
    coarse.size = aggregates;
    // every coupling between two different aggregates, as (from, to) pairs, sorted and
    // unique: the coarse CSR in row order with ascending columns
    std::vector<std::pair<std::uint32_t, std::uint32_t>> couplings;
    couplings.reserve(fine.column.size());
    for (std::uint32_t row = 0; row < fine.size; ++row) {
        for (std::uint32_t k = fine.offset[row]; k < fine.offset[row + 1]; ++k) {
            if (agg[fine.column[k]] != agg[row]) couplings.emplace_back(agg[row], agg[fine.column[k]]);
        }
    }
    std::sort(couplings.begin(), couplings.end());
    couplings.erase(std::unique(couplings.begin(), couplings.end()), couplings.end());
    coarse.offset.assign(aggregates + 1, 0);
    coarse.column.resize(couplings.size());
    for (std::size_t e = 0; e < couplings.size(); ++e) {
        ++coarse.offset[couplings[e].first + 1];
        coarse.column[e] = couplings[e].second;
    }
    for (std::uint32_t a = 0; a < aggregates; ++a) {
        coarse.width = std::max(coarse.width, coarse.offset[a + 1]);
        coarse.offset[a + 1] += coarse.offset[a];
    }
    coarse.diagonal.assign(aggregates, 0.0);
    coarse.value.assign(coarse.column.size(), 0.0);
    // where each fine off-diagonal lands: per aggregate, its coarse columns' positions
    // marked in a scratch row, read back by every member's entries
    fine.target.assign(fine.column.size(), -1);
    std::vector<std::uint32_t> start, rows;
    members_of(agg, aggregates, start, rows);
    std::vector<std::int64_t> position(aggregates, -1);
    for (std::uint32_t a = 0; a < aggregates; ++a) {
        for (std::uint32_t e = coarse.offset[a]; e < coarse.offset[a + 1]; ++e) position[coarse.column[e]] = e;
        for (std::uint32_t m = start[a]; m < start[a + 1]; ++m) {
            const std::uint32_t row = rows[m];
            for (std::uint32_t k = fine.offset[row]; k < fine.offset[row + 1]; ++k) {
                const std::uint32_t to = agg[fine.column[k]];
                if (to != a) fine.target[k] = position[to];
            }
        }
        for (std::uint32_t e = coarse.offset[a]; e < coarse.offset[a + 1]; ++e) position[coarse.column[e]] = -1;
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
