// Host driver: planet upload, batch layout, V-cycle and Krylov orchestration.
//
// A batch concatenates planets level by level. Planet i's rows on level l occupy
// [base_l[i], base_l[i] + n_il), padded to whole 256-row tiles, so that every tile
// belongs to one planet: per-planet dot products, convergence and gating are then
// decided per tile. A one-planet batch is the drop-in solve of the reference's
// solve_newton_system/GraphMultigrid (sim/planet/surface/heat_transport.cpp:337-429,
// 545-577); a many-planet batch solves uneven planets with the same launches.
#include "solver.hpp"

#include "kernels.hpp"
#include "coarse_tail.hpp"
#include "host/agglomerate.hpp"
#include "host/shared_columns.hpp"
#include "krylov.hpp"
#include "persistent.hpp"
#include "profile.hpp"

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace psgb {

namespace {

// Levels with at least this many tiles (two waves of eight 256-thread blocks on 152 SMs)
// use multi-tile sets by default.
constexpr std::uint32_t kSetsMinTiles = 2 * 8 * 152;

// Levels whose planets hold at most this many rows each run in the coarse tail.
constexpr std::uint32_t kTailRows = 4096;

template <typename T>
void upload_to(T* dst, const std::vector<T>& host) {
    if (!host.empty()) PSGB_CUDA(cudaMemcpy(dst, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
}

}  // namespace

// Tile sets pay where a level has several waves of 256-row blocks; small levels need
// every block they can get.
void default_launch_shapes(Batch& b) {
    for (BatchLevel& L : b.levels) {
        L.sets_stencil = L.tiles >= kSetsMinTiles ? 2 : 1;
        L.sets_vector = L.tiles >= kSetsMinTiles ? 4 : 1;
    }
    b.tail_level = b.default_tail_level;
}

std::unique_ptr<Planet> make_planet(std::uint32_t level, double radius_m, bool agglomerated) {
    auto planet = std::make_unique<Planet>();
    if (agglomerated && level > 0) {
        // The transport one level coarser: the coarse mesh's graph, nodes taking the
        // areas of the fine cells that join them (heat_transport.cpp:467-512).
        const HostMesh fine = build_icosphere(level, radius_m);
        planet->mesh = build_icosphere(level - 1, radius_m);
        planet->graph = transport_graph(planet->mesh);
        Agglomeration agg = agglomerate(fine, planet->mesh);
        planet->graph.area_m2 = std::move(agg.area_m2);
        planet->group_of_cell = std::move(agg.group_of_cell);
        planet->member_offset = std::move(agg.member_offset);
        planet->member = std::move(agg.member);
        planet->fine_area_m2 = std::move(agg.fine_area_m2);
        planet->fine_cells = fine.cells;
    } else {
        planet->mesh = build_icosphere(level, radius_m);
        planet->graph = transport_graph(planet->mesh);
        if (agglomerated) {   // level 0: the mesh itself
            Agglomeration agg = identity_agglomeration(planet->mesh);
            planet->group_of_cell = std::move(agg.group_of_cell);
            planet->member_offset = std::move(agg.member_offset);
            planet->member = std::move(agg.member);
            planet->fine_area_m2 = std::move(agg.fine_area_m2);
            planet->fine_cells = planet->mesh.cells;
        }
    }
    planet->hierarchy = build_hierarchy(planet->graph);
    for (const auto& lv : planet->hierarchy.levels) {
        if (lv.width > 16) throw std::logic_error("hierarchy level wider than 16");
    }
    if (planet->hierarchy.levels.back().size > coarsest_rows) {
        throw std::logic_error("coarsest multigrid level exceeds 400 rows");
    }
    return planet;
}

void upload_planet(Planet& planet_ref) {
    if (planet_ref.uploaded) return;
    Planet* planet = &planet_ref;
    // Operator geometry (finite_volume.cpp:34-111), ELL slot-major over P rows.
    const HostMesh& m = planet->mesh;
    DevMesh& d = planet->dev;
    d.n = static_cast<std::uint32_t>(m.cells);
    d.p = pad_rows(d.n);
    d.edges = static_cast<std::uint32_t>(m.edges);
    const std::size_t P = d.p;
    std::vector<std::int32_t> nbr(6 * P), edge(6 * P, 0);
    std::vector<std::uint8_t> first(P, 0), degree(P, 0);
    std::vector<double> w(6 * P, 0.0), dist(6 * P, 1.0), area(P, 1.0), gm(4 * P, 0.0);
    std::vector<float> ne(6 * P, 0.0F), nn(6 * P, 0.0F);
    for (std::size_t r = 0; r < P; ++r)
        for (int j = 0; j < 6; ++j) nbr[j * P + r] = static_cast<std::int32_t>(r);
    for (std::size_t c = 0; c < m.cells; ++c) {
        const std::uint32_t base = m.edge_offset[c];
        degree[c] = m.edge_count[c];
        area[c] = m.area_m2[c];
        double mee = 0.0, men = 0.0, mnn = 0.0;
        for (std::uint32_t k = 0; k < m.edge_count[c]; ++k) {
            const std::uint32_t e = m.nb_edge[base + k];
            nbr[k * P + c] = static_cast<std::int32_t>(m.nb_cell[base + k]);
            edge[k * P + c] = static_cast<std::int32_t>(e);
            if (m.edge_first[e] == c) first[c] |= static_cast<std::uint8_t>(1u << k);
            w[k * P + c] = planet->graph.weight[base + k];
            dist[k * P + c] = m.edge_distance_m[e];
            ne[k * P + c] = m.normal_east[base + k];
            nn[k * P + c] = m.normal_north[base + k];
            const double a = static_cast<double>(m.normal_east[base + k]);
            const double b = static_cast<double>(m.normal_north[base + k]);
            mee += a * a;
            men += a * b;
            mnn += b * b;
        }
        gm[0 * P + c] = mee;
        gm[1 * P + c] = men;
        gm[2 * P + c] = mnn;
        gm[3 * P + c] = mee * mnn - men * men;
    }
    d.nbr = planet->store.upload(nbr);
    d.edge = planet->store.upload(edge);
    d.first = planet->store.upload(first);
    d.degree = planet->store.upload(degree);
    d.w = planet->store.upload(w);
    d.dist = planet->store.upload(dist);
    d.ne = planet->store.upload(ne);
    d.nn = planet->store.upload(nn);
    d.area = planet->store.upload(area);
    {
        std::vector<double> graph_area(P, 1.0);
        for (std::size_t c = 0; c < m.cells; ++c) graph_area[c] = planet->graph.area_m2[c];
        d.graph_area = planet->store.upload(graph_area);
    }
    if (!planet->group_of_cell.empty()) {
        d.fine_cells = static_cast<std::uint32_t>(planet->fine_cells);
        d.group_of_cell = planet->store.upload(planet->group_of_cell);
        d.member_offset = planet->store.upload(planet->member_offset);
        d.member = planet->store.upload(planet->member);
        d.fine_area = planet->store.upload(planet->fine_area_m2);
    }
    d.gm = planet->store.upload(gm);
    {   // sin(lat) = z, cos(lat) = sqrt(x^2 + y^2) as the reference forms them
        std::vector<double> latitude(2 * P, 0.0);
        for (std::size_t c = 0; c < m.cells; ++c) {
            const double x = m.center[3 * c], y = m.center[3 * c + 1];
            latitude[c] = m.center[3 * c + 2];
            latitude[P + c] = std::sqrt(x * x + y * y);
        }
        d.latitude = planet->store.upload(latitude);
    }
    d.edge_length = planet->store.upload(m.edge_length_m);
    planet->uploaded = true;
}

namespace {
std::unique_ptr<Batch> build_batch(const std::vector<Planet*>& planets, void* arena, std::size_t arena_bytes);
}  // namespace

std::unique_ptr<Batch> make_batch(const std::vector<Planet*>& planets) {
    return build_batch(planets, nullptr, 0);
}

std::unique_ptr<Batch> make_batch_in(const std::vector<Planet*>& planets, void* arena, std::size_t arena_bytes) {
    if (arena == nullptr) throw std::invalid_argument("no scratch memory given");
    return build_batch(planets, arena, arena_bytes);
}

namespace {

// The fine level's columns once per distinct graph (host/shared_columns.hpp): a batch of
// many planets of one mesh level streams one small copy (L2-resident) instead of one copy
// a planet. The level's own `col` stays for the kernels that read it (assembly, coarse
// tails).
void share_columns(BatchLevel& L, const std::vector<Planet*>& planets, const std::vector<std::int32_t>& tile_inst,
                   DeviceStore& store) {
    std::vector<const HostLevel*> fine(planets.size());
    for (std::size_t i = 0; i < planets.size(); ++i) fine[i] = &planets[i]->hierarchy.levels[0];
    const SharedColumns s = shared_columns(fine, L.base, tile_inst, L.width);
    if (s.pitch == 0) return;
    std::vector<int2> shift(tile_inst.size());
    for (std::size_t t = 0; t < shift.size(); ++t) shift[t] = make_int2(s.shift[2 * t], s.shift[2 * t + 1]);
    L.scol = store.upload(s.scol);
    L.tile_shift = store.upload(shift);
    L.spitch = s.pitch;
}

std::unique_ptr<Batch> build_batch(const std::vector<Planet*>& planets, void* arena, std::size_t arena_bytes) {
    if (planets.empty()) throw std::invalid_argument("a batch needs at least one planet");
    if (planets.size() >= kMaxInstances) throw std::invalid_argument("a batch holds fewer than 4,194,304 planets");
    if (arena == nullptr) {
        for (Planet* p : planets) upload_planet(*p);
    }
    auto bp = std::make_unique<Batch>();
    Batch& b = *bp;
    if (arena != nullptr) {
        b.store.use_arena(arena, arena_bytes);
        b.use_graphs = false;
    }
    b.planets = planets;
    b.instances = static_cast<std::uint32_t>(planets.size());
    const std::uint32_t I = b.instances;
    std::size_t depth = 0;
    for (auto* p : planets) depth = std::max(depth, p->hierarchy.levels.size());
    b.levels.resize(depth);

    // Row bases, tiles and widths per level.
    for (std::size_t l = 0; l < depth; ++l) {
        BatchLevel& L = b.levels[l];
        L.base.assign(I, -1);
        L.count.assign(I, 0);
        std::uint32_t rows = 0, width = 0;
        for (std::uint32_t i = 0; i < I; ++i) {
            const auto& H = planets[i]->hierarchy.levels;
            if (l >= H.size()) continue;
            L.base[i] = rows;
            L.count[i] = H[l].size;
            rows += pad_rows(H[l].size);
            width = std::max(width, H[l].width);
        }
        L.rows = rows;
        L.tiles = rows / kTileRows;
        L.width = device_width(std::max<std::uint32_t>(width, 1));
        if (l == 0) L.width = 6;
    }
    b.fine_base = b.levels[0].base;
    // Per planet and level: its tile range; the coarse tail starts at the first level
    // where no planet holds more than kTailRows rows.
    {
        std::vector<std::uint32_t> range(depth * I * 2, 0u);
        for (std::size_t l = 0; l < depth; ++l) {
            for (std::uint32_t i = 0; i < I; ++i) {
                if (b.levels[l].base[i] < 0) continue;
                range[(l * I + i) * 2] = static_cast<std::uint32_t>(b.levels[l].base[i] / kTileRows);
                range[(l * I + i) * 2 + 1] = pad_rows(b.levels[l].count[i]) / kTileRows;
            }
        }
        b.tile_range = b.store.upload(range);
        for (std::size_t l = 1; l < depth && b.default_tail_level == 0; ++l) {
            std::uint32_t most = 0;
            for (std::uint32_t i = 0; i < I; ++i) most = std::max(most, b.levels[l].count[i]);
            if (most <= kTailRows) b.default_tail_level = static_cast<int>(l);
        }
    }
    default_launch_shapes(b);

    // Tile metadata and ELL columns.
    for (std::size_t l = 0; l < depth; ++l) {
        BatchLevel& L = b.levels[l];
        const std::size_t P = L.rows, W = L.width;
        std::vector<std::int32_t> tile_inst(L.tiles), tile_rows(L.tiles);
        std::vector<std::uint8_t> tile_sweep(L.tiles);
        std::vector<std::int32_t> col(W * P);
        for (std::size_t r = 0; r < P; ++r)
            for (std::size_t j = 0; j < W; ++j) col[j * P + r] = static_cast<std::int32_t>(r);
        for (std::uint32_t i = 0; i < I; ++i) {
            if (L.base[i] < 0) continue;
            const auto& H = planets[i]->hierarchy.levels;
            const HostLevel& hl = H[l];
            const std::uint32_t t0 = static_cast<std::uint32_t>(L.base[i] / kTileRows);
            const std::uint32_t nt = pad_rows(hl.size) / kTileRows;
            for (std::uint32_t t = 0; t < nt; ++t) {
                tile_inst[t0 + t] = static_cast<std::int32_t>(i);
                tile_rows[t0 + t] = static_cast<std::int32_t>(std::min<std::uint32_t>(kTileRows, hl.size - t * kTileRows));
                tile_sweep[t0 + t] = (l + 1 < H.size()) ? 1 : 0;
            }
            for (std::uint32_t r = 0; r < hl.size; ++r) {
                for (std::uint32_t k = hl.offset[r]; k < hl.offset[r + 1]; ++k) {
                    col[(k - hl.offset[r]) * P + L.base[i] + r] = static_cast<std::int32_t>(L.base[i] + hl.column[k]);
                }
            }
        }
        L.tile_inst = b.store.upload(tile_inst);
        L.tile_rows = b.store.upload(tile_rows);
        L.tile_sweep = b.store.upload(tile_sweep);
        // packed per-tile word for the solve phases, padded to whole groups of four tiles
        std::vector<std::uint32_t> meta((L.tiles + 3) / 4 * 4, 0u);
        for (std::uint32_t t = 0; t < L.tiles; ++t) meta[t] = pack_tile(tile_inst[t], tile_rows[t], tile_sweep[t] != 0);
        L.tile_meta = b.store.upload(meta);

        L.col = b.store.upload(col);
        if (l == 0 && arena == nullptr && I > 1) share_columns(L, planets, tile_inst, b.store);
        L.vd64 = b.store.alloc<double>((W + 1) * P);
        L.vd32 = b.store.alloc<float>((W + 1) * P);
        L.inv64 = b.store.alloc<double>(P);
        L.inv32 = b.store.alloc<float>(P);
        PSGB_CUDA(cudaMemset(L.vd64, 0, (W + 1) * P * sizeof(double)));
        L.x64 = b.store.alloc<double>(P); L.y64 = b.store.alloc<double>(P);
        L.b64 = b.store.alloc<double>(P); L.r64 = b.store.alloc<double>(P);
        L.x32 = b.store.alloc<float>(P); L.y32 = b.store.alloc<float>(P);
        L.b32 = b.store.alloc<float>(P); L.r32 = b.store.alloc<float>(P);
        for (double* v : {L.x64, L.y64, L.b64, L.r64}) PSGB_CUDA(cudaMemset(v, 0, P * sizeof(double)));
        for (float* v : {L.x32, L.y32, L.b32, L.r32}) PSGB_CUDA(cudaMemset(v, 0, P * sizeof(float)));
    }

    // Level transitions: aggregates, restriction members, Galerkin gather lists.
    for (std::size_t l = 0; l + 1 < depth; ++l) {
        BatchLevel& F = b.levels[l];
        BatchLevel& C = b.levels[l + 1];
        const std::size_t Pf = F.rows, Wf = F.width, Pc = C.rows, Wc = C.width;
        // Rows without an aggregate may be loaded through but never store: a planet's padding
        // rows point at its own first coarse row, so that every load stays within the
        // planet's rows (the shared-memory tails hold only those); rows of planets whose
        // coarsest level this is point at coarse row 0.
        std::vector<std::int32_t> agg(Pf, 0);
        std::vector<std::vector<std::uint32_t>> members(Pc);
        std::vector<std::vector<std::uint32_t>> lists((Wc + 1) * Pc);
        for (std::uint32_t i = 0; i < I; ++i) {
            if (C.base[i] < 0) continue;
            const HostLevel& hf = planets[i]->hierarchy.levels[l];
            const HostLevel& hc = planets[i]->hierarchy.levels[l + 1];
            const std::int64_t bf = F.base[i], bc = C.base[i];
            for (std::uint32_t r = hf.size; r < pad_rows(hf.size); ++r) agg[bf + r] = static_cast<std::int32_t>(bc);
            for (std::uint32_t r = 0; r < hf.size; ++r) {
                const std::uint32_t a = hf.aggregate[r];
                const std::size_t gr = bf + r, ga = bc + a;
                agg[gr] = static_cast<std::int32_t>(ga);
                members[ga].push_back(static_cast<std::uint32_t>(gr));
                lists[Wc * Pc + ga].push_back(static_cast<std::uint32_t>(Wf * Pf + gr));
                for (std::uint32_t k = hf.offset[r]; k < hf.offset[r + 1]; ++k) {
                    const std::uint32_t src = static_cast<std::uint32_t>((k - hf.offset[r]) * Pf + gr);
                    if (hf.target[k] < 0) {
                        lists[Wc * Pc + ga].push_back(src);
                    } else {
                        const std::uint32_t j = static_cast<std::uint32_t>(hf.target[k]) - hc.offset[a];
                        lists[j * Pc + ga].push_back(src);
                    }
                }
            }
        }
        std::vector<std::uint32_t> moff(Pc + 1, 0), mem;
        for (std::size_t a = 0; a < Pc; ++a) {
            mem.insert(mem.end(), members[a].begin(), members[a].end());
            moff[a + 1] = static_cast<std::uint32_t>(mem.size());
        }
        std::vector<std::uint32_t> goff(lists.size() + 1, 0), gsrc;
        for (std::size_t id = 0; id < lists.size(); ++id) {
            gsrc.insert(gsrc.end(), lists[id].begin(), lists[id].end());
            goff[id + 1] = static_cast<std::uint32_t>(gsrc.size());
        }
        F.agg = b.store.upload(agg);
        F.member_offset = b.store.upload(moff);
        F.member = b.store.upload(mem);
        F.gal_offset = b.store.upload(goff);
        F.gal_source = b.store.upload(gsrc);
        F.gal_lists = static_cast<std::uint32_t>(lists.size());
    }

    // Coarsest levels: dense inverses.
    DenseCoarse& D = b.dense;
    D.level.resize(I); D.offset.resize(I); D.size.resize(I); D.row_base.resize(I);
    std::uint64_t total = 0;
    for (std::uint32_t i = 0; i < I; ++i) {
        const auto& H = planets[i]->hierarchy.levels;
        const int c = static_cast<int>(H.size()) - 1;
        D.level[i] = c;
        D.size[i] = H[c].size;
        D.offset[i] = total;
        D.row_base[i] = b.levels[c].base[i];
        D.max_rows = std::max(D.max_rows, H[c].size);
        total += std::uint64_t(H[c].size) * H[c].size;
    }
    b.dense_at.assign(depth, 0);
    for (std::uint32_t i = 0; i < I; ++i) b.dense_at[static_cast<std::size_t>(D.level[i])] = 1;
    std::vector<int2> blocks;
    D.block_offset.assign(depth + 1, 0);
    for (std::size_t l = 0; l < depth; ++l) {
        D.block_offset[l] = static_cast<std::uint32_t>(blocks.size());
        for (std::uint32_t i = 0; i < I; ++i) {
            if (D.level[i] != static_cast<int>(l)) continue;
            for (std::uint32_t r = 0; r < D.size[i]; r += 8) blocks.push_back(int2{static_cast<int>(i), static_cast<int>(r)});
        }
    }
    D.block_offset[depth] = static_cast<std::uint32_t>(blocks.size());
    D.d_blocks = b.store.upload(blocks);
    D.inv64 = b.store.alloc<double>(total);
    D.inv32 = b.store.alloc<float>(total);
    D.work = b.store.alloc<double>(total);
    D.d_level = b.store.upload(D.level);
    D.d_offset = b.store.upload(D.offset);
    D.d_size = b.store.upload(D.size);
    D.d_row_base = b.store.upload(D.row_base);

    // Fine-level graph data and Krylov workspace.
    const BatchLevel& F = b.levels[0];
    const std::size_t P0 = F.rows;
    std::vector<double> area(P0, 1.0), w(6 * P0, 0.0), wsum(P0, 0.0);
    std::vector<std::uint32_t> tile_begin(I + 1, 0);
    for (std::uint32_t i = 0; i < I; ++i) {
        const TransportGraph& g = planets[i]->graph;
        const std::int64_t base = F.base[i];
        for (std::size_t c = 0; c < g.size(); ++c) {
            area[base + c] = g.area_m2[c];
            wsum[base + c] = g.weight_sum[c];
            for (std::uint32_t k = g.offset[c]; k < g.offset[c + 1]; ++k) {
                w[(k - g.offset[c]) * P0 + base + c] = g.weight[k];
            }
        }
        tile_begin[i] = static_cast<std::uint32_t>(base / kTileRows);
    }
    tile_begin[I] = F.tiles;
    b.area = b.store.upload(area);
    b.w = b.store.upload(w);
    b.wsum = b.store.upload(wsum);
    b.conductance = b.store.alloc<double>(I);
    for (int v = 0; v < Batch::kVectors; ++v) {
        b.k64[v] = b.store.alloc<double>(P0);
        b.k32[v] = b.store.alloc<float>(P0);
        PSGB_CUDA(cudaMemset(b.k64[v], 0, P0 * sizeof(double)));
        PSGB_CUDA(cudaMemset(b.k32[v], 0, P0 * sizeof(float)));
    }
    b.xr = b.store.alloc<double>(P0);
    b.rr = b.store.alloc<double>(P0);
    b.bb = b.store.alloc<double>(P0);
    b.tmp = b.store.alloc<double>(P0);
    b.tmp2 = b.store.alloc<double>(P0);
    for (double* v : {b.xr, b.rr, b.bb, b.tmp, b.tmp2}) PSGB_CUDA(cudaMemset(v, 0, P0 * sizeof(double)));
    b.partial = b.store.alloc<double>(std::size_t(F.tiles) * 8);
    b.ticket = b.store.alloc<unsigned>(I);
    PSGB_CUDA(cudaMemset(b.ticket, 0, I * sizeof(unsigned)));
    b.sync = b.store.alloc<unsigned>(4);
    PSGB_CUDA(cudaMemset(b.sync, 0, 4 * sizeof(unsigned)));
    // The coarse tail's blocks per planet for every possible tail level, laid out now so
    // that no allocation happens while a stream records (one block each where the
    // device cannot hold every planet's blocks at once).
    {
        const unsigned budget = tail_block_budget();
        b.tail_cta_at.assign(depth, nullptr);
        b.tail_ctas_at.assign(depth, 0u);
        for (std::size_t l = 1; l < depth && budget >= I; ++l) {
            std::vector<std::uint32_t> rows(I, 0);
            for (std::uint32_t i = 0; i < I; ++i)
                if (b.levels[l].base[i] >= 0) rows[i] = b.levels[l].count[i];
            const std::vector<std::uint32_t> cta = tail_blocks(rows, budget);
            if (cta.size() > I) {
                b.tail_cta_at[l] = b.store.upload(cta);
                b.tail_ctas_at[l] = static_cast<unsigned>(cta.size());
            }
        }
        // the shared-memory tail's rows per tail level (largest planet)
        b.tail_rows_at.assign(depth, 0u);
        for (std::size_t l = 1; l < depth; ++l) {
            for (std::uint32_t i = 0; i < I; ++i) {
                unsigned rows = 0;
                for (std::size_t k = l; k < depth && b.levels[k].base[i] >= 0; ++k) rows += pad_rows(b.levels[k].count[i]);
                b.tail_rows_at[l] = std::max(b.tail_rows_at[l], rows);
            }
        }
        b.tail_barrier = b.store.alloc<unsigned>(2 * std::size_t(I));
        PSGB_CUDA(cudaMemset(b.tail_barrier, 0, 2 * std::size_t(I) * sizeof(unsigned)));
    }
    b.tile_begin = b.store.upload(tile_begin);
    b.scalars = b.store.alloc<InstanceScalars>(I);
    PSGB_CUDA(cudaMemset(b.scalars, 0, I * sizeof(InstanceScalars)));
    b.host_scalars.assign(I, InstanceScalars{});
    if (arena == nullptr) PSGB_CUDA(cudaMallocHost(&b.pinned_scalars, I * sizeof(InstanceScalars)));
    b.slope_of = b.store.alloc<double>(I);
    b.t0 = b.store.alloc<double>(P0);
    b.src = b.store.alloc<double>(P0);
    b.hout = b.store.alloc<double>(P0);
    b.tnew = b.store.alloc<double>(P0);
    for (double* v : {b.t0, b.src, b.hout, b.tnew}) PSGB_CUDA(cudaMemset(v, 0, P0 * sizeof(double)));
    b.sums = b.store.alloc<double>(std::size_t(I) * 8);
    b.active = b.store.alloc<std::uint8_t>(I);
    PSGB_CUDA(cudaMemset(b.active, 1, I));
    b.host_active.assign(I, 1);
    if (arena == nullptr) {
        PSGB_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
        PSGB_CUDA(cudaEventCreateWithFlags(&b.fence_in, cudaEventDisableTiming));
        PSGB_CUDA(cudaEventCreateWithFlags(&b.fence_out, cudaEventDisableTiming));
    }
    if (I == 1) b.csr_offset = b.store.upload(planets[0]->graph.offset);
    return bp;
}

}  // namespace

template <typename T>
static LevelView<T> make_view(const BatchLevel& L, const T* vd, const T* inv, std::size_t level) {
    LevelView<T> v{L.rows,         L.width,        L.tiles,      L.col,
                   vd,             inv,            L.tile_inst,  L.tile_rows,
                   L.tile_sweep,   L.tile_meta,    nullptr,
                   L.sets_stencil, L.sets_vector,  static_cast<std::uint8_t>(level)};
    v.scol = L.scol;
    v.tile_shift = L.tile_shift;
    v.spitch = L.spitch;
    return v;
}

template <typename T>
bool tail_fits_shared(const Batch& b, int level) {
    if (level <= 0 || static_cast<std::size_t>(level) >= b.tail_rows_at.size()) return false;
    return std::size_t(4) * b.tail_rows_at[level] * sizeof(T) <= tail_shared_max_bytes<T>();
}
template bool tail_fits_shared<float>(const Batch&, int);
template bool tail_fits_shared<double>(const Batch&, int);

unsigned tail_cluster_rows(const Batch& b, int level, unsigned cluster) {
    if (level <= 0 || static_cast<std::size_t>(level) >= b.levels.size() || cluster == 0) return 0;
    unsigned most = 0;
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        unsigned rows = 0;
        for (std::size_t k = static_cast<std::size_t>(level); k < b.levels.size() && b.levels[k].base[i] >= 0; ++k) {
            const unsigned tiles = pad_rows(b.levels[k].count[i]) / kTileRows;
            rows += (tiles + cluster - 1) / cluster * kTileRows;
        }
        most = std::max(most, rows);
    }
    return most;
}

template <typename T>
bool tail_fits_cluster(const Batch& b, int level, unsigned cluster) {
    const unsigned rows = tail_cluster_rows(b, level, cluster);
    return rows != 0 && cluster_tail_fits<T>(cluster, rows);
}
template bool tail_fits_cluster<float>(const Batch&, int, unsigned);
template bool tail_fits_cluster<double>(const Batch&, int, unsigned);

template <typename T>
TailForm tail_form(const Batch& b) {
    if (b.tail_level <= 0) return TailForm::kNone;
    if (b.tail_cluster != 0 && tail_fits_cluster<T>(b, b.tail_level, b.tail_cluster)) return TailForm::kCluster;
    if (b.tail_shared && tail_fits_shared<T>(b, b.tail_level)) return TailForm::kShared;
    if (b.tail_spread && b.tail_cta_at[b.tail_level] != nullptr) return TailForm::kSpread;
    return TailForm::kBlock;
}
template TailForm tail_form<float>(const Batch&);
template TailForm tail_form<double>(const Batch&);

StepView step_view(const Batch& b) {
    const BatchLevel& F = b.levels[0];
    return StepView{F.rows, F.tiles, b.instances, F.tile_inst, F.tile_rows, b.tile_begin, F.col, b.w, b.area,
                    b.conductance, b.step_edge_conductance, b.slope_of, profile_bytes_for(kFamStep)};
}

LevelView<double> view64(const Batch& b, std::size_t level) {
    const BatchLevel& L = b.levels[level];
    LevelView<double> v = make_view<double>(L, L.vd64, L.inv64, level);
    v.correction = b.smoother.correction;
    return v;
}

LevelView<float> view32(const Batch& b, std::size_t level) {
    const BatchLevel& L = b.levels[level];
    LevelView<float> v = make_view<float>(L, L.vd32, L.inv32, level);
    v.correction = static_cast<float>(b.smoother.correction);
    return v;
}

namespace {

template <typename T>
struct Pick;
template <>
struct Pick<double> {
    static LevelView<double> view(const Batch& b, std::size_t l) { return view64(b, l); }
    static double* x(BatchLevel& L) { return L.x64; }
    static double* y(BatchLevel& L) { return L.y64; }
    static double* bvec(BatchLevel& L) { return L.b64; }
    static double* r(BatchLevel& L) { return L.r64; }
    static const double* inv(const DenseCoarse& D) { return D.inv64; }
    static double** k(Batch& b) { return b.k64; }
};
template <>
struct Pick<float> {
    static LevelView<float> view(const Batch& b, std::size_t l) { return view32(b, l); }
    static float* x(BatchLevel& L) { return L.x32; }
    static float* y(BatchLevel& L) { return L.y32; }
    static float* bvec(BatchLevel& L) { return L.b32; }
    static float* r(BatchLevel& L) { return L.r32; }
    static const float* inv(const DenseCoarse& D) { return D.inv32; }
    static float** k(Batch& b) { return b.k32; }
};

DenseView dense_view(const Batch& b) {
    const DenseCoarse& D = b.dense;
    return DenseView{b.instances, D.d_level, D.d_offset, D.d_size, D.d_row_base};
}

// The dense solves of the planets whose coarsest level is `level`.
template <typename T>
DenseTask<T> dense_task(Batch& b, std::size_t level, const T* rhs, T* x) {
    const DenseCoarse& D = b.dense;
    const std::uint32_t begin = D.block_offset[level], end = D.block_offset[level + 1];
    return DenseTask<T>{dense_view(b), D.d_blocks + begin, end - begin, Pick<T>::inv(D), rhs, x};
}

template <typename T>
PersistentLevel<T> level_of(Batch& b, std::size_t l) {
    BatchLevel& L = b.levels[l];
    return PersistentLevel<T>{Pick<T>::view(b, l), Pick<T>::x(L), Pick<T>::y(L), Pick<T>::bvec(L), Pick<T>::r(L),
                              L.member_offset, L.member, L.agg};
}

template <typename T>
TailArgs<T> tail_args(Batch& b, int gate) {
    TailArgs<T> a{};
    const std::size_t depth = b.levels.size();
    if (depth > static_cast<std::size_t>(kMaxLevels)) throw std::logic_error("coarse tail: hierarchy deeper than 12 levels");
    for (std::size_t l = 0; l < depth; ++l) {
        a.level[l] = level_of<T>(b, l);
        a.level[l].view.bytes = profile_bytes_for(kFamSmoothCoarse);
        a.pre[l] = b.smoother.pre_at(l);
        a.post[l] = b.smoother.post_at(l);
        a.inner[l] = b.smoother.inner_at(l);
        a.starts_in_x[l] = b.smoother.starts_in_x(l) ? 1 : 0;
    }
    a.tile_range = b.tile_range;
    a.first = b.tail_level;
    a.depth = static_cast<int>(depth);
    a.instances = b.instances;
    a.dense = dense_view(b);
    a.dense_inv = Pick<T>::inv(b.dense);
    a.omega = static_cast<T>(b.smoother.omega);
    a.sc = b.scalars;
    a.gate = gate;
    a.shared_rows = 0;
    a.cluster = 0;
    const TailForm form = tail_form<T>(b);
    b.tail_launch_blocks = b.instances;
    if (form == TailForm::kCluster) {
        a.cluster = b.tail_cluster;
        a.shared_rows = tail_cluster_rows(b, b.tail_level, b.tail_cluster);
        a.error = b.sync + 3;
        b.tail_launch_blocks = b.instances * b.tail_cluster;
        return a;
    }
    if (form == TailForm::kShared) {
        a.shared_rows = b.tail_rows_at[b.tail_level];
        return a;
    }
    // Per-planet blocks in proportion to the planets' rows at the tail level.
    if (form == TailForm::kSpread) {
        a.cta = b.tail_cta_at[b.tail_level];
        a.ctas = b.tail_ctas_at[b.tail_level];
        a.barrier = b.tail_barrier;
        a.error = b.sync + 3;
        b.tail_launch_blocks = a.ctas;
    }
    return a;
}

}  // namespace

void assemble_transport(Batch& b, const double* slope, const double* conductance,
                        const double* edge_conductance, cudaStream_t st) {
    const LevelView<double> fine = view64(b, 0);
    launch_assemble_transport(fine, b.w, b.wsum, b.area, slope, conductance, edge_conductance,
                              b.levels[0].vd64, st);
}

void set_matrix_csr(Batch& b, const double* diag, const double* off, cudaStream_t st) {
    if (b.instances != 1) throw std::invalid_argument("set_matrix applies to a one-planet batch");
    Planet& p = *b.planets[0];
    launch_set_matrix_csr(static_cast<std::uint32_t>(p.graph.size()), b.levels[0].rows, b.levels[0].width,
                          b.csr_offset, diag, off, b.levels[0].vd64, st);
}

void prepare_levels(Batch& b, cudaStream_t st) {
    for (std::size_t l = 0; l + 1 < b.levels.size(); ++l) {
        BatchLevel& F = b.levels[l];
        BatchLevel& C = b.levels[l + 1];
        launch_galerkin(F.gal_lists, F.gal_offset, F.gal_source, F.vd64, C.vd64, st);
    }
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        BatchLevel& L = b.levels[l];
        launch_finalize_level(L.rows, L.width, L.vd64, L.vd32, L.inv64, L.inv32, st);
    }
    const DenseView dv = dense_view(b);
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        bool any = false;
        for (auto c : b.dense.level) any = any || (c == static_cast<int>(l));
        if (!any) continue;
        launch_dense_invert(dv, static_cast<int>(l), view64(b, l), b.dense.work, b.dense.inv64,
                            b.dense.inv32, st);
    }
    PSGB_CUDA(cudaGetLastError());
    b.matrix_ready = true;
}

template <typename T>
T* vcycle_first_target(Batch& b, T* x) {
    return b.smoother.starts_in_x(0) ? x : Pick<T>::y(b.levels[0]);
}

template <typename T>
void vcycle(Batch& b, const T* rhs, T* x, int gate, bool first_sweep_done, cudaStream_t st) {
    const std::size_t depth = b.levels.size();
    const SmootherConfig& sm = b.smoother;
    const T omega = static_cast<T>(sm.omega);
    std::vector<T*> cur(depth), other(depth);
    std::vector<const T*> rhs_of(depth);
    for (std::size_t l = 0; l < depth; ++l) {
        BatchLevel& L = b.levels[l];
        T* X = (l == 0) ? x : Pick<T>::x(L);
        T* Y = Pick<T>::y(L);
        cur[l] = sm.starts_in_x(l) ? X : Y;
        other[l] = sm.starts_in_x(l) ? Y : X;
        rhs_of[l] = (l == 0) ? rhs : Pick<T>::bvec(L);
    }
    // Levels from `tail` down run as one block per planet (0: none).
    const std::size_t tail =
        (b.tail_level > 0 && static_cast<std::size_t>(b.tail_level) < depth) ? static_cast<std::size_t>(b.tail_level) : 0;
    const std::size_t down_end = tail != 0 ? tail : depth - 1;
    // Planets whose only level is the fine one: dense solve there.
    if (b.dense_at[0]) launch_dense_solve<T>(dense_task<T>(b, 0, rhs, x), b.scalars, gate, st);
    // Down: pre-smoothing, residual, restriction fused with the next level's first sweep.
    for (std::size_t l = 0; l < down_end; ++l) {
        const LevelView<T> lv = Pick<T>::view(b, l);
        BatchLevel& L = b.levels[l];
        // Planets whose coarsest level is this one (l >= 1) solve it in extra blocks of the
        // level's first launch: they do not smooth here, the others do not need them yet.
        DenseTask<T> dense{};
        if (l > 0 && b.dense_at[l]) dense = dense_task<T>(b, l, Pick<T>::bvec(L), Pick<T>::x(L));
        if (l == 0 && !first_sweep_done) launch_smooth_zero<T>(lv, rhs_of[l], cur[l], omega, b.scalars, gate, st);
        for (int k = 1; k < sm.pre_at(l); ++k) {
            launch_smooth<T>(lv, rhs_of[l], cur[l], other[l], omega, b.scalars, gate, st, dense, sm.inner_at(l));
            dense = DenseTask<T>{};
            std::swap(cur[l], other[l]);
        }
        BatchLevel& C = b.levels[l + 1];
        const LevelView<T> cv = Pick<T>::view(b, l + 1);
        if (l > 0) {
            // coarse levels: latency-bound, the residual formed inside the restriction (on
            // the fine level, HBM-bound, the warp-per-coarse-row gathers of the members'
            // rows cost more than the residual's own pass: 11.1 -> 12.7 ms on the 64-planet
            // step, 8.7 -> 11.3 ms on one L8 planet in FP64)
            launch_residual_restrict<T>(lv, cv, L.member_offset, L.member, rhs_of[l], cur[l], Pick<T>::bvec(C),
                                        cur[l + 1], omega, b.scalars, gate, st, dense);
        } else {
            launch_residual<T>(lv, rhs_of[l], cur[l], Pick<T>::r(L), b.scalars, gate, st, dense);
            launch_restrict_zero<T>(cv, L.member_offset, L.member, Pick<T>::r(L), Pick<T>::bvec(C), cur[l + 1], omega,
                                    b.scalars, gate, st);
        }
        // The deepest level has no smoothing launch: its dense solves run on their own.
        if (tail == 0 && l + 2 == depth && b.dense_at[l + 1]) {
            launch_dense_solve<T>(dense_task<T>(b, l + 1, Pick<T>::bvec(C), Pick<T>::x(C)), b.scalars, gate, st);
        }
    }
    if (tail != 0) launch_coarse_tail<T>(tail_args<T>(b, gate), st);
    // Up: prolongation fused with the first post-smoothing sweep.
    for (std::size_t l = tail != 0 ? tail : depth - 1; l-- > 0;) {
        const LevelView<T> lv = Pick<T>::view(b, l);
        BatchLevel& L = b.levels[l];
        const T* e = Pick<T>::x(b.levels[l + 1]);
        // FP64 on the fine level: the fused prolongation adds the correction to every
        // neighbour it reads (7 more FP64 additions a row), and GB300's FP64 pipe, not
        // HBM, would bound the sweep; add it once in its own pass instead (same sums,
        // same bits). FP32 and the latency-bound coarse levels keep the fused launch.
        const bool split = std::is_same<T, double>::value && l == 0;
        if (sm.post_at(l) == 0 || split) {
            launch_prolong<T>(lv, L.agg, e, cur[l], b.scalars, gate, st);
            for (int k = 0; k < sm.post_at(l); ++k) {
                launch_smooth<T>(lv, rhs_of[l], cur[l], other[l], omega, b.scalars, gate, st, DenseTask<T>{},
                                 sm.inner_at(l));
                std::swap(cur[l], other[l]);
            }
            continue;
        }
        launch_prolong_smooth<T>(lv, L.agg, e, rhs_of[l], cur[l], other[l], omega, b.scalars, gate, st);
        std::swap(cur[l], other[l]);
        for (int k = 1; k < sm.post_at(l); ++k) {
            launch_smooth<T>(lv, rhs_of[l], cur[l], other[l], omega, b.scalars, gate, st, DenseTask<T>{}, sm.inner_at(l));
            std::swap(cur[l], other[l]);
        }
    }
}

template void vcycle<double>(Batch&, const double*, double*, int, bool, cudaStream_t);
template void vcycle<float>(Batch&, const float*, float*, int, bool, cudaStream_t);
template double* vcycle_first_target<double>(Batch&, double*);
template float* vcycle_first_target<float>(Batch&, float*);

namespace {

ReduceCtx reduce_ctx(Batch& b) { return ReduceCtx{b.partial, b.ticket, b.tile_begin, b.scalars, b.instances}; }

// What a recorded Krylov chunk depends on besides precision, method and length: the
// per-level sweeps and launch shapes.
std::vector<int> shape_of(const Batch& b) {
    std::vector<int> shape;
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        shape.push_back(b.smoother.pre_at(l));
        shape.push_back(b.smoother.post_at(l));
        shape.push_back(b.smoother.inner_at(l));
        shape.push_back(b.levels[l].sets_stencil);
        shape.push_back(b.levels[l].sets_vector);
    }
    shape.push_back(b.tail_level);
    shape.push_back(b.tail_spread ? 1 : 0);
    shape.push_back(b.tail_shared ? 1 : 0);
    shape.push_back(static_cast<int>(b.tail_cluster));
    return shape;
}

bool all_done(Batch& b, cudaStream_t st, bool outer) {
    InstanceScalars* host = b.pinned_scalars != nullptr ? b.pinned_scalars : b.host_scalars.data();
    PSGB_CUDA(cudaMemcpyAsync(host, b.scalars, b.instances * sizeof(InstanceScalars), cudaMemcpyDeviceToHost, st));
    PSGB_CUDA(cudaStreamSynchronize(st));
    for (std::uint32_t i = 0; i < b.instances; ++i) {
        const InstanceScalars& s = host[i];
        if (outer ? s.outer_status == kRunning : (s.outer_status == kRunning && s.status == kRunning)) return false;
    }
    return true;
}

// One chunk of `count` Krylov iterations (BiCGSTAB or PCG), all launches on `st`.
template <typename T>
void krylov_chunk(Batch& b, int method, int count, T* rhs_unused, T* x, cudaStream_t st) {
    static_cast<void>(rhs_unused);
    using K = KrylovLaunch<T>;
    const LevelView<T> lv = Pick<T>::view(b, 0);
    const ReduceCtx ctx = reduce_ctx(b);
    T** v = Pick<T>::k(b);
    const T omega_j = static_cast<T>(b.smoother.omega);
    for (int k = 0; k < count; ++k) {
        if (method == kBiCGSTAB) {
            T *r = v[0], *shadow = v[1], *p = v[2], *vv = v[3], *phat = v[4], *s = v[5], *shat = v[6], *t = v[7];
            K::bicg_p(lv, r, vv, p, vcycle_first_target<T>(b, phat), omega_j, b.scalars, st);
            vcycle<T>(b, p, phat, kGateRunning, true, st);
            K::bicg_v(lv, phat, vv, shadow, ctx, st);
            K::bicg_s(lv, r, vv, s, vcycle_first_target<T>(b, shat), omega_j, ctx, st);
            vcycle<T>(b, s, shat, kGateSecondHalf, true, st);
            K::bicg_t(lv, shat, t, s, ctx, st);
            K::bicg_x(lv, phat, shat, s, t, x, r, shadow, ctx, st);
        } else {
            T *r = v[0], *p = v[2], *q = v[3], *z = v[4];
            K::pcg_rz(lv, r, z, ctx, st);
            K::pcg_p(lv, z, p, b.scalars, st);
            K::pcg_q(lv, p, q, ctx, st);
            K::pcg_xr(lv, p, q, x, r, vcycle_first_target<T>(b, z), omega_j, ctx, st);
            vcycle<T>(b, r, z, kGateRunning, true, st);
        }
    }
}

// The chunk as a CUDA graph, recorded once per (precision, method, chunk, smoother).
template <typename T>
GraphEntry& chunk_graph(Batch& b, int method, int count, T* x, cudaStream_t st) {
    const GraphKey key{static_cast<int>(sizeof(T)), method, count, shape_of(b), b.smoother.omega,
                       b.smoother.correction};
    GraphEntry& g = b.graphs[key];
    if (g.exec != nullptr) return g;
    cudaGraph_t graph = nullptr;
    set_capturing(true);
    PSGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        krylov_chunk<T>(b, method, count, nullptr, x, st);
    } catch (...) {
        cudaStreamEndCapture(st, &graph);
        set_capturing(false);
        if (graph != nullptr) cudaGraphDestroy(graph);
        throw;
    }
    const cudaError_t end = cudaStreamEndCapture(st, &graph);
    set_capturing(false);
    PSGB_CUDA(end);
    std::size_t nodes = 0;
    PSGB_CUDA(cudaGraphGetNodes(graph, nullptr, &nodes));
    const cudaError_t inst = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    PSGB_CUDA(inst);
    g.kernels = nodes;
    return g;
}

// Inner Krylov solve A x = rhs (level-0 vectors in T), x0 = 0.
template <typename T>
void krylov(Batch& b, const SolveOptions& opt, const T* rhs, T* x, double tol, cudaStream_t st) {
    using K = KrylovLaunch<T>;
    const LevelView<T> lv = Pick<T>::view(b, 0);
    const ReduceCtx ctx = reduce_ctx(b);
    T** v = Pick<T>::k(b);
    const T omega_j = static_cast<T>(b.smoother.omega);
    const int max_it = opt.max_iterations;
    if (opt.method == kBiCGSTAB) {
        K::bicg_init(lv, rhs, x, v[0], v[1], v[2], v[3], ctx, tol, max_it, st);
    } else {
        K::pcg_init(lv, rhs, x, v[0], v[2], vcycle_first_target<T>(b, v[4]), omega_j, ctx, tol, max_it, st);
        vcycle<T>(b, v[0], v[4], kGateRunning, true, st);
    }
    const bool graphs = b.use_graphs && !profile_active();
    int it = 0;
    while (it < max_it) {
        const int count = std::min(opt.poll, max_it - it);
        if (graphs) {
            GraphEntry& g = chunk_graph<T>(b, opt.method, count, x, st);
            PSGB_CUDA(cudaGraphLaunch(g.exec, st));
            count_graph_kernels(g.kernels);
        } else {
            krylov_chunk<T>(b, opt.method, count, nullptr, x, st);
        }
        it += count;
        PSGB_CUDA(cudaGetLastError());
        if (all_done(b, st, false)) break;
    }
}

// Arguments of the persistent solve: the same vectors, views and scalars the kernel path
// passes launch by launch.
template <typename T>
PersistentArgs<T> persistent_args(Batch& b, const SolveOptions& opt, const double* rhs, double* x, double inner_tol) {
    PersistentArgs<T> a{};
    a.depth = static_cast<int>(b.levels.size());
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        a.level[l] = level_of<T>(b, l);
        a.dense_at[l] = b.dense_at[l] ? 1 : 0;
    }
    for (std::size_t l = 0; l < b.levels.size(); ++l) a.level[l].view.bytes = profile_bytes_for(kFamPersistent);
    a.dense = dense_view(b);
    a.dense_inv = Pick<T>::inv(b.dense);
    a.dense_blocks = b.dense.d_blocks;
    for (std::size_t l = 0; l <= b.levels.size(); ++l) a.dense_block_offset[l] = b.dense.block_offset[l];
    a.fine64 = view64(b, 0);
    a.rhs64 = rhs;
    a.x64 = x;
    a.r64 = b.rr;
    for (int k = 0; k < Batch::kVectors; ++k) a.k[k] = Pick<T>::k(b)[k];
    a.ctx = reduce_ctx(b);
    a.sc = b.scalars;
    a.instances = b.instances;
    a.active = b.active_mask ? b.active : nullptr;
    a.tolerance = opt.tolerance;
    a.inner_tolerance = inner_tol;
    a.max_iterations = opt.max_iterations;
    a.max_refinements = opt.max_refinements;
    a.method = opt.method;
    for (std::size_t l = 0; l < b.levels.size(); ++l) {
        a.pre[l] = b.smoother.pre_at(l);
        a.post[l] = b.smoother.post_at(l);
        a.inner[l] = b.smoother.inner_at(l);
        a.starts_in_x[l] = b.smoother.starts_in_x(l) ? 1 : 0;
    }
    a.omega = static_cast<T>(b.smoother.omega);
    a.sync = PersistentSync{b.sync, b.sync + 1, b.sync + 2};
    return a;
}

// The automatic schedule is the kernel schedule: on GB300 its many resident blocks hide
// the latency of the small per-tile phases better than one 1024-thread block per SM.
bool use_persistent(const Batch& b, const SolveOptions& opt) {
    if (opt.schedule != kSchedulePersistent) return false;
    if (b.levels.size() > static_cast<std::size_t>(kMaxLevels))
        throw std::invalid_argument("persistent schedule: hierarchy deeper than 12 levels");
    if (!persistent_supported()) throw std::runtime_error("persistent schedule: the device cannot run it");
    return true;
}

}  // namespace

void solve(Batch& b, const SolveOptions& opt, const double* rhs, double* x, cudaStream_t caller) {
    if (!b.matrix_ready) throw std::logic_error("solve before the matrix was set");
    // The solve runs on the batch's own stream (capturable), ordered after the caller's
    // work and before anything the caller enqueues next.
    cudaStream_t st = b.stream != nullptr ? b.stream : caller;
    if (b.stream != nullptr) {
        PSGB_CUDA(cudaEventRecord(b.fence_in, caller));
        PSGB_CUDA(cudaStreamWaitEvent(st, b.fence_in, 0));
    }
    const LevelView<double> lv64 = view64(b, 0);
    const ReduceCtx ctx = reduce_ctx(b);
    const bool persistent = use_persistent(b, opt);
    // Inner target: max(inner_tol * ||r||, tolerance * ||b|| / 2); the plain FP64 solve
    // reaches the outer target in one refinement, the mixed one in a few.
    const double inner_tol = opt.precision == kMixed ? opt.inner_tolerance : 1e-3 * opt.tolerance;
    if (!persistent) {
        launch_outer_init(lv64, rhs, ctx, opt.tolerance, opt.max_refinements, b.active_mask ? b.active : nullptr, st);
    } else {
        // The whole refinement loop in one cooperative launch (outer_init included).
        PSGB_CUDA(cudaMemsetAsync(b.sync, 0, 4 * sizeof(unsigned), st));
        if (opt.precision == kMixed) {
            launch_persistent<float>(persistent_args<float>(b, opt, rhs, x, inner_tol), st, b.stream != nullptr);
        } else {
            launch_persistent<double>(persistent_args<double>(b, opt, rhs, x, inner_tol), st, b.stream != nullptr);
        }
    }
    for (int refine = 0; !persistent && refine <= opt.max_refinements; ++refine) {
        if (opt.precision == kMixed) {
            launch_outer_residual<float>(lv64, rhs, x, b.rr, b.k32[8], ctx, opt.max_refinements, st);
        } else {
            launch_outer_residual<double>(lv64, rhs, x, b.rr, b.k64[8], ctx, opt.max_refinements, st);
        }
        if (all_done(b, st, true)) break;
        if (opt.precision == kMixed) {
            krylov<float>(b, opt, b.k32[8], b.k32[9], inner_tol, st);
            launch_outer_update<float>(lv64, b.k32[9], x, b.scalars, b.instances, st);
        } else {
            krylov<double>(b, opt, b.k64[8], b.k64[9], inner_tol, st);
            launch_outer_update<double>(lv64, b.k64[9], x, b.scalars, b.instances, st);
        }
    }
    InstanceScalars* host = b.pinned_scalars != nullptr ? b.pinned_scalars : b.host_scalars.data();
    PSGB_CUDA(cudaMemcpyAsync(host, b.scalars, b.instances * sizeof(InstanceScalars), cudaMemcpyDeviceToHost, st));
    unsigned barrier_error[2] = {0, 0};
    const TailForm form = persistent ? TailForm::kNone
                                     : (opt.precision == kMixed ? tail_form<float>(b) : tail_form<double>(b));
    if (persistent || form == TailForm::kSpread || form == TailForm::kCluster) {
        PSGB_CUDA(cudaMemcpyAsync(barrier_error, b.sync + 2, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    }
    PSGB_CUDA(cudaStreamSynchronize(st));
    if (barrier_error[0] != 0) {
        throw std::runtime_error("persistent solve: a grid-barrier wait ran past its iteration limit");
    }
    if (barrier_error[1] != 0) {
        // the per-planet barriers' state is unknown after a timeout: start them afresh
        PSGB_CUDA(cudaMemset(b.tail_barrier, 0, 2 * std::size_t(b.instances) * sizeof(unsigned)));
        PSGB_CUDA(cudaMemset(b.sync + 3, 0, sizeof(unsigned)));
        if (form == TailForm::kCluster)
            throw std::runtime_error("coarse tail: a row index fell outside its planet's slices of the cluster");
        throw std::runtime_error("coarse tail: a per-planet barrier wait ran past its limit");
    }
    if (host != b.host_scalars.data()) {
        std::memcpy(b.host_scalars.data(), host, b.instances * sizeof(InstanceScalars));
    }
    if (b.stream != nullptr) {
        PSGB_CUDA(cudaEventRecord(b.fence_out, st));
        PSGB_CUDA(cudaStreamWaitEvent(caller, b.fence_out, 0));
    }
}

}  // namespace psgb
