// Host check of the block ILU(0) structure (planet_game_gb300/csrc/host/ilu_pattern.cpp),
// compiled and run by tests/test_ilu_pattern_host.py: on random symmetric patterns with
// random blocks, (1) every row appears once in each level schedule and the rows a row
// depends on sit in earlier levels of its block; (2) replaying the IKJ update list level
// by level, in any order within a level, gives the same factor, bit for bit, as the plain
// sequential IKJ elimination of incomplete_lu.cpp:108-135 restated here; (3) the
// shared-memory records list each row's couplings in the factor's order.
#include "host/ilu_pattern.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <set>
#include <vector>

using namespace psgb;

static int fail(const char* what, int trial) {
    std::printf("FAIL %s (trial %d)\n", what, trial);
    return 1;
}

int main() {
    std::mt19937_64 rng(20261203);
    for (int trial = 0; trial < 40; ++trial) {
        const std::uint32_t n = 50 + rng() % 400;
        std::vector<std::set<std::uint32_t>> adj(n);
        const std::uint32_t edges = n * (2 + rng() % 3);
        for (std::uint32_t e = 0; e < edges; ++e) {
            const std::uint32_t a = rng() % n, b = (a + 1 + rng() % 12) % n;   // local-ish couplings
            if (a != b) { adj[a].insert(b); adj[b].insert(a); }
        }
        std::vector<std::uint32_t> offset{0}, neighbour;
        for (std::uint32_t i = 0; i < n; ++i) {
            std::vector<std::uint32_t> row(adj[i].begin(), adj[i].end());
            std::shuffle(row.begin(), row.end(), rng);                  // CSR order need not be sorted
            neighbour.insert(neighbour.end(), row.begin(), row.end());
            offset.push_back(static_cast<std::uint32_t>(neighbour.size()));
        }
        std::vector<std::uint32_t> blocks{0};
        while (blocks.back() < n) blocks.push_back(std::min<std::uint32_t>(n, blocks.back() + 1 + rng() % 90));
        const IluPattern p = ilu_pattern(offset, neighbour, blocks);
        // (1) schedules
        for (const LevelSchedule* s : {&p.lower, &p.upper}) {
            std::vector<int> seen(n, 0), level_of(n, -1);
            for (std::uint32_t b = 0; b + 1 < blocks.size(); ++b)
                for (std::uint32_t lv = s->block_level[b]; lv < s->block_level[b + 1]; ++lv)
                    for (std::uint32_t idx = s->level_start[lv]; idx < s->level_start[lv + 1]; ++idx) {
                        const std::uint32_t i = s->order[idx];
                        if (i < blocks[b] || i >= blocks[b + 1]) return fail("row outside its block", trial);
                        ++seen[i];
                        level_of[i] = static_cast<int>(lv);
                    }
            for (std::uint32_t i = 0; i < n; ++i)
                if (seen[i] != 1) return fail("row not scheduled exactly once", trial);
            const bool lower = s == &p.lower;
            for (std::uint32_t i = 0; i < n; ++i) {
                const std::uint32_t q0 = lower ? p.start[i] : p.diagonal[i] + 1;
                const std::uint32_t q1 = lower ? p.diagonal[i] : p.start[i + 1];
                for (std::uint32_t q = q0; q < q1; ++q)
                    if (level_of[p.column[q]] >= level_of[i]) return fail("dependency not in an earlier level", trial);
            }
        }
        // (2) the factor: sequential IKJ against the update list replayed level by level
        std::vector<double> diag(n), off(neighbour.size());
        std::uniform_real_distribution<double> u(-1.0, 0.0);
        for (auto& v : off) v = u(rng);
        for (std::uint32_t i = 0; i < n; ++i) diag[i] = 8.0 + 4.0 * (rng() % 1000) / 1000.0;
        std::vector<double> value(p.column.size());
        for (std::uint32_t i = 0; i < n; ++i)
            for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q)
                value[q] = p.source[q] < 0 ? diag[i] : off[p.source[q]];
        std::vector<double> seq = value, lvl = value;
        for (std::uint32_t b = 0; b + 1 < blocks.size(); ++b) {     // sequential IKJ, rows in order
            const std::uint32_t first = blocks[b], last = blocks[b + 1];
            std::vector<long> position(last - first, -1);
            for (std::uint32_t i = first; i < last; ++i) {
                for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q) position[p.column[q] - first] = q;
                for (std::uint32_t q = p.start[i]; q < p.diagonal[i]; ++q) {
                    const std::uint32_t j = p.column[q];
                    seq[q] /= seq[p.diagonal[j]];
                    for (std::uint32_t t = p.diagonal[j] + 1; t < p.start[j + 1]; ++t) {
                        const long at = position[p.column[t] - first];
                        if (at >= 0) seq[at] -= seq[q] * seq[t];
                    }
                }
                for (std::uint32_t q = p.start[i]; q < p.start[i + 1]; ++q) position[p.column[q] - first] = -1;
            }
        }
        for (std::uint32_t b = 0; b + 1 < blocks.size(); ++b) {     // level by level, rows reversed in a level
            for (std::uint32_t lv = p.lower.block_level[b]; lv < p.lower.block_level[b + 1]; ++lv) {
                for (std::uint32_t idx = p.lower.level_start[lv + 1]; idx-- > p.lower.level_start[lv];) {
                    const std::uint32_t i = p.lower.order[idx];
                    for (std::uint32_t q = p.start[i]; q < p.diagonal[i]; ++q) {
                        const double lq = lvl[q] / lvl[p.diagonal[p.column[q]]];
                        lvl[q] = lq;
                        for (std::uint32_t k = p.update_start[q]; k < p.update_start[q + 1]; ++k)
                            lvl[p.update_at[k]] -= lq * lvl[p.update_t[k]];
                    }
                }
            }
        }
        for (std::size_t q = 0; q < seq.size(); ++q)
            if (seq[q] != lvl[q]) return fail("level-scheduled factor differs from the sequential one", trial);
        // (3) records
        if (!p.lower.rec_row.empty()) {
            for (const LevelSchedule* s : {&p.lower, &p.upper}) {
                const bool lower = s == &p.lower;
                for (std::uint32_t b = 0; b + 1 < blocks.size(); ++b)
                    for (std::uint32_t lv = s->block_level[b]; lv < s->block_level[b + 1]; ++lv)
                        for (std::uint32_t idx = s->level_start[lv]; idx < s->level_start[lv + 1]; ++idx) {
                            const std::uint32_t i = s->order[idx];
                            if (s->rec_row[idx] != i - blocks[b]) return fail("record row", trial);
                            const std::uint32_t q0 = lower ? p.start[i] : p.diagonal[i] + 1;
                            const std::uint32_t q1 = lower ? p.diagonal[i] : p.start[i + 1];
                            if (s->rec_count[idx] != q1 - q0) return fail("record count", trial);
                            for (std::uint32_t q = q0; q < q1; ++q) {
                                if (s->rec_q[std::size_t(idx) * kIluRecord + (q - q0)] != q) return fail("record value position", trial);
                                if (s->rec_col[std::size_t(idx) * kIluRecord + (q - q0)] != p.column[q] - blocks[b])
                                    return fail("record column", trial);
                            }
                        }
            }
        }
    }
    std::printf("OK\n");
    return 0;
}
