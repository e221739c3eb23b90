// Host check of the shared fine-level columns (planet_game_gb300/csrc/host/
// shared_columns.cpp), run by tests/test_shared_columns_host.py: for a batch whose planets
// repeat two graphs and hold one of their own, every column of every row (valid or
// padding, every slot) read through a tile's shift from the shared copy equals the
// per-planet ELL column the batch builds; the copy holds each distinct graph once; a
// batch with no repeated graph shares nothing.
#include "host/shared_columns.hpp"

#include <cstdio>
#include <vector>

using namespace psgb;

static int fail(const char* what) {
    std::printf("FAIL %s\n", what);
    return 1;
}

// A CSR graph of n rows with 3..6 neighbours a row (a few rows short, as pentagons are).
static HostLevel graph(std::uint32_t n, std::uint32_t seed) {
    HostLevel h;
    h.size = n;
    h.offset.push_back(0);
    std::uint32_t state = seed;
    for (std::uint32_t r = 0; r < n; ++r) {
        state = state * 1664525u + 1013904223u;
        const std::uint32_t degree = 3 + (state >> 28) % 4;
        for (std::uint32_t k = 0; k < degree; ++k) {
            state = state * 1664525u + 1013904223u;
            h.column.push_back((r + 1 + (state >> 8) % (n - 1)) % n);
        }
        h.offset.push_back(static_cast<std::uint32_t>(h.column.size()));
    }
    return h;
}

// The per-planet ELL columns as the batch lays them out: slot-major over P rows, a row's
// own index in missing slots and padding rows.
static std::vector<std::int32_t> ell(const std::vector<const HostLevel*>& fine, const std::vector<std::int64_t>& base,
                                     std::size_t P, std::size_t W) {
    std::vector<std::int32_t> col(W * P);
    for (std::size_t r = 0; r < P; ++r)
        for (std::size_t j = 0; j < W; ++j) col[j * P + r] = static_cast<std::int32_t>(r);
    for (std::size_t i = 0; i < fine.size(); ++i) {
        const HostLevel& h = *fine[i];
        for (std::uint32_t r = 0; r < h.size; ++r)
            for (std::uint32_t k = h.offset[r]; k < h.offset[r + 1]; ++k)
                col[(k - h.offset[r]) * P + base[i] + r] = static_cast<std::int32_t>(base[i] + h.column[k]);
    }
    return col;
}

static int check(const std::vector<const HostLevel*>& fine, bool shared_expected, std::uint32_t pitch_expected) {
    const std::size_t W = 6;
    std::vector<std::int64_t> base;
    std::vector<std::int32_t> tile_inst;
    std::int64_t rows = 0;
    for (std::size_t i = 0; i < fine.size(); ++i) {
        base.push_back(rows);
        for (std::uint32_t t = 0; t < pad_rows(fine[i]->size) / 256; ++t) tile_inst.push_back(static_cast<std::int32_t>(i));
        rows += pad_rows(fine[i]->size);
    }
    const std::size_t P = static_cast<std::size_t>(rows);
    const std::vector<std::int32_t> col = ell(fine, base, P, W);
    const SharedColumns s = shared_columns(fine, base, tile_inst, W);
    if (!shared_expected) return s.pitch == 0 ? 0 : fail("a batch without repeated graphs shared columns");
    if (s.pitch != pitch_expected) return fail("the shared copy does not hold each distinct graph once");
    if (s.scol.size() != W * s.pitch || s.shift.size() != 2 * tile_inst.size()) return fail("array sizes");
    for (std::size_t t = 0; t < tile_inst.size(); ++t) {
        for (std::size_t lane = 0; lane < 256; ++lane) {
            const std::int64_t row = static_cast<std::int64_t>(t * 256 + lane);
            const std::int64_t local = row - s.shift[2 * t + 1];
            if (local < 0 || local >= s.pitch) return fail("a row reads outside the shared copy");
            for (std::size_t j = 0; j < W; ++j) {
                const std::int64_t c = s.shift[2 * t] + s.scol[j * s.pitch + static_cast<std::size_t>(local)];
                if (c != col[j * P + static_cast<std::size_t>(row)]) return fail("a shared column differs");
            }
        }
    }
    return 0;
}

int main() {
    const HostLevel a = graph(600, 1), b = graph(300, 2), c = graph(300, 3), d = graph(1000, 4);
    // a and b repeated (b and c of equal size but different graphs), d on its own
    if (int e = check({&a, &b, &a, &c, &a, &b, &d}, true, 768 + 512 + 512 + 1024)) return e;
    if (int e = check({&b, &b}, true, 512)) return e;
    if (int e = check({&a, &b, &c, &d}, false, 0)) return e;
    if (int e = check({&d}, false, 0)) return e;
    std::printf("OK\n");
    return 0;
}
