// Host-side spherical centroidal Voronoi mesh builder.
//
// Produces, bit for bit, the mesh of the reference builder make_icosphere
// (sim/planet/mesh/icosphere.cpp:200-419): icosahedron subdivision with 20 Lloyd
// iterations per level (:92-118, :225-259), recursive face order -> cell order
// (:265-279), circumcentre corners (:76-83, :284-292), per-cell corner order by
// atan2 in the local east/north basis with index tie-break (:322-335), Kahan-summed
// cell areas (:339-352), edge ids in order of first appearance (:361-388) and FP32
// outward normals (:64-71, :390-395).
//
// Unlike the reference, the Lloyd accumulation and the per-cell geometry run on
// all host cores. Every per-vertex sum keeps the reference's order (faces in
// ascending order, "next" neighbour before "previous"), so the result does not
// depend on the thread count. Edge ids come from one ordered pass: an edge is new
// exactly when it is met from its lower-numbered cell, because cells are visited
// in ascending order.
#include "mesh.hpp"
#include "parallel.hpp"
#include "vec3.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <map>
#include <memory>
#include <mutex>
#include <unordered_map>

namespace psgb {
namespace {

using Face = std::array<std::uint32_t, 3>;

constexpr std::uint32_t lloyd_iterations = 20;

double triangle_area_unit(const V3& a, const V3& b, const V3& c) {
    const double num = std::abs(dot(a, cross(b, c)));
    const double den = 1.0 + dot(a, b) + dot(b, c) + dot(c, a);
    return 2.0 * std::atan2(num, den);
}

double arc(const V3& a, const V3& b) { return std::acos(std::clamp(dot(a, b), -1.0, 1.0)); }

V3 circumcentre(const V3& a, const V3& b, const V3& c) {
    V3 centre = unit(cross(sub(b, a), sub(c, a)));
    if (dot(centre, add(add(a, b), c)) < 0.0) {
        centre = scale(centre, -1.0);
    }
    return centre;
}

V3 outward_normal(const V3& centre, const V3& c1, const V3& c2) {
    V3 conormal = unit(cross(c1, c2));
    if (dot(conormal, centre) > 0.0) {
        conormal = scale(conormal, -1.0);
    }
    return unit(sub(conormal, scale(centre, dot(conormal, centre))));
}

std::vector<V3> icosahedron_vertices() {
    const double g = 1.6180339887498948482;
    const double raw[12][3] = {{-1, g, 0}, {1, g, 0},   {-1, -g, 0}, {1, -g, 0},
                               {0, -1, g}, {0, 1, g},   {0, -1, -g}, {0, 1, -g},
                               {g, 0, -1}, {g, 0, 1},   {-g, 0, -1}, {-g, 0, 1}};
    std::vector<V3> v;
    for (const auto& r : raw) v.push_back(unit(V3{r[0], r[1], r[2]}));
    return v;
}

std::vector<Face> icosahedron_faces() {
    return {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
            {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
            {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
            {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
}

// vertex -> incident faces in ascending face order, with the vertex's corner slot.
struct Incidence {
    std::vector<std::uint32_t> offset, face;
    std::vector<std::uint8_t> slot;
};

Incidence incidence(std::size_t vertices, const std::vector<Face>& faces) {
    Incidence inc;
    inc.offset.assign(vertices + 1, 0);
    for (const auto& f : faces)
        for (auto v : f) ++inc.offset[v + 1];
    for (std::size_t v = 0; v < vertices; ++v) inc.offset[v + 1] += inc.offset[v];
    inc.face.resize(inc.offset.back());
    inc.slot.resize(inc.offset.back());
    std::vector<std::uint32_t> fill(inc.offset.begin(), inc.offset.end() - 1);
    for (std::size_t f = 0; f < faces.size(); ++f) {
        for (std::uint8_t s = 0; s < 3; ++s) {
            const auto v = faces[f][s];
            inc.face[fill[v]] = static_cast<std::uint32_t>(f);
            inc.slot[fill[v]] = s;
            ++fill[v];
        }
    }
    return inc;
}

// Lloyd relaxation towards the centroidal tessellation, as the reference's
// Jacobi-style update (icosphere.cpp:92-118), with its per-vertex sum order. Each
// iteration computes the faces' circumcentres, then every vertex sums the two
// area-weighted centroids of each incident face's corner (faces in ascending order,
// "next" neighbour before "previous") from the old positions into a second buffer.
void lloyd(std::vector<V3>& v, const std::vector<Face>& faces, std::uint32_t iterations) {
    const Incidence inc = incidence(v.size(), faces);
    std::vector<V3> centre(faces.size()), next(v.size());
    for (std::uint32_t it = 0; it < iterations; ++it) {
        parallel_for(faces.size(), [&](std::size_t f) {
            const Face& face = faces[f];
            centre[f] = circumcentre(v[face[0]], v[face[1]], v[face[2]]);
        });
        parallel_for(v.size(), [&](std::size_t vertex) {
            const V3& gen = v[vertex];
            V3 sum{0.0, 0.0, 0.0};
            for (std::uint32_t k = inc.offset[vertex]; k < inc.offset[vertex + 1]; ++k) {
                const Face& face = faces[inc.face[k]];
                const V3& cc = centre[inc.face[k]];
                const std::size_t c = inc.slot[k];
                for (std::size_t side = 1; side <= 2; ++side) {
                    const V3 mid = unit(add(gen, v[face[(c + side) % 3]]));
                    const double area = triangle_area_unit(gen, mid, cc);
                    sum = add(sum, scale(unit(add(add(gen, mid), cc)), area));
                }
            }
            next[vertex] = unit(sum);
        });
        v.swap(next);
    }
}

struct UnitMesh {
    std::vector<V3> vertices;
    std::vector<Face> faces;
};

// One level finer: every face split in four at its edges' normalised midpoints (a
// midpoint is numbered when first met, faces in order), then the Lloyd relaxation.
void subdivide_and_relax(UnitMesh& u) {
    std::vector<V3>& vert = u.vertices;
    std::vector<Face>& faces = u.faces;
    std::unordered_map<std::uint64_t, std::uint32_t> midpoints;
    midpoints.reserve(faces.size() * 2);
    auto midpoint = [&](std::uint32_t a, std::uint32_t b) {
        const std::uint64_t key = (std::uint64_t(std::min(a, b)) << 32) | std::max(a, b);
        auto it = midpoints.find(key);
        if (it != midpoints.end()) return it->second;
        const auto index = static_cast<std::uint32_t>(vert.size());
        vert.push_back(unit(add(vert[a], vert[b])));
        midpoints.emplace(key, index);
        return index;
    };
    std::vector<Face> next;
    next.reserve(faces.size() * 4);
    for (const auto& f : faces) {
        const auto e01 = midpoint(f[0], f[1]);
        const auto e12 = midpoint(f[1], f[2]);
        const auto e20 = midpoint(f[2], f[0]);
        next.push_back({f[0], e01, e20});
        next.push_back({f[1], e12, e01});
        next.push_back({f[2], e20, e12});
        next.push_back({e01, e12, e20});
    }
    faces.swap(next);
    lloyd(vert, faces, lloyd_iterations);
}

// The relaxed unit mesh of `level`, built once per process from the finest level
// already built below it; every level passed on the way is kept too (a level's mesh
// depends only on the level, so an L8 build leaves L1-L7 ready).
const UnitMesh& relaxed_unit_mesh(std::uint32_t level) {
    static std::mutex mutex;
    static std::map<std::uint32_t, std::unique_ptr<UnitMesh>> cache;
    std::unique_lock<std::mutex> lock(mutex);
    if (const auto hit = cache.find(level); hit != cache.end()) return *hit->second;
    UnitMesh u;
    std::uint32_t from = 0;
    if (auto below = cache.lower_bound(level); below != cache.begin()) {
        --below;
        u = *below->second;
        from = below->first;
    } else {
        u.vertices = icosahedron_vertices();
        u.faces = icosahedron_faces();
    }
    lock.unlock();
    for (std::uint32_t l = from; l < level; ++l) {
        subdivide_and_relax(u);
        if (l + 1 < level) {
            auto copy = std::make_unique<UnitMesh>(u);
            lock.lock();
            auto& entry = cache[l + 1];
            if (!entry) entry = std::move(copy);
            lock.unlock();
        }
    }
    auto built = std::make_unique<UnitMesh>(std::move(u));
    lock.lock();
    auto& entry = cache[level];
    if (!entry) entry = std::move(built);
    return *entry;
}

}  // namespace

std::size_t icosphere_cell_count(std::uint32_t level) {
    if (level > 13) throw std::overflow_error("icosphere level too large for 32-bit ids");
    return 10u * (std::size_t(1) << (2 * level)) + 2u;
}

HostMesh build_icosphere(std::uint32_t level, double radius_m) {
    if (!(radius_m > 0.0) || !std::isfinite(radius_m)) {
        throw std::invalid_argument("icosphere radius must be finite and positive");
    }
    const std::size_t n_cells = icosphere_cell_count(level);
    const std::size_t n_faces = 20u * (std::size_t(1) << (2 * level));

    // The relaxed unit-sphere mesh depends on the level only; the radius enters the
    // final geometry. It is built once per level and cached for the process.
    const UnitMesh& unit_mesh = relaxed_unit_mesh(level);
    const std::vector<V3>& vert = unit_mesh.vertices;
    const std::vector<Face>& faces = unit_mesh.faces;
    if (faces.size() != n_faces || vert.size() != n_cells) {
        throw std::logic_error("icosphere subdivision produced unexpected counts");
    }

    // Cell order: first appearance in the recursive face order.
    constexpr auto none = std::numeric_limits<std::uint32_t>::max();
    std::vector<std::uint32_t> cell_of(vert.size(), none), source_of;
    source_of.reserve(n_cells);
    for (const auto& f : faces) {
        for (auto s : f) {
            if (cell_of[s] == none) {
                cell_of[s] = static_cast<std::uint32_t>(source_of.size());
                source_of.push_back(s);
            }
        }
    }

    HostMesh m;
    m.level = level;
    m.radius_m = radius_m;
    m.cells = n_cells;
    m.corners = n_faces;
    m.directed = 6 * n_cells - 12;
    m.edges = 3 * n_cells - 6;
    m.corner_unit.resize(3 * n_faces);
    std::vector<V3> corner(n_faces);
    parallel_for(n_faces, [&](std::size_t f) {
        corner[f] = circumcentre(vert[faces[f][0]], vert[faces[f][1]], vert[faces[f][2]]);
        m.corner_unit[3 * f] = corner[f].x;
        m.corner_unit[3 * f + 1] = corner[f].y;
        m.corner_unit[3 * f + 2] = corner[f].z;
    });
    const Incidence inc = incidence(vert.size(), faces);

    // Local basis per cell (sim/planet/coordinates/local_tangent_basis.cpp:8-24).
    std::vector<V3> up(n_cells), east(n_cells), north(n_cells);
    m.center.resize(3 * n_cells);
    m.east.resize(3 * n_cells);
    m.north.resize(3 * n_cells);
    m.source_vertex = source_of;
    m.edge_count.resize(n_cells);
    m.edge_offset.resize(n_cells);
    parallel_for(n_cells, [&](std::size_t c) {
        const V3 u = unit(vert[source_of[c]]);
        const double h = std::hypot(u.x, u.y);
        const V3 e = h > 1.0e-12 ? V3{-u.y / h, u.x / h, 0.0} : V3{0.0, 1.0, 0.0};
        const V3 n = unit(cross(u, e));
        up[c] = u;
        east[c] = e;
        north[c] = n;
        m.center[3 * c] = u.x; m.center[3 * c + 1] = u.y; m.center[3 * c + 2] = u.z;
        m.east[3 * c] = e.x; m.east[3 * c + 1] = e.y; m.east[3 * c + 2] = e.z;
        m.north[3 * c] = n.x; m.north[3 * c + 1] = n.y; m.north[3 * c + 2] = n.z;
        const std::uint32_t deg = inc.offset[source_of[c] + 1] - inc.offset[source_of[c]];
        if (deg != 5 && deg != 6) throw std::logic_error("dual cell is neither a pentagon nor a hexagon");
        m.edge_count[c] = static_cast<std::uint8_t>(deg);
    });
    std::uint32_t running = 0;
    for (std::size_t c = 0; c < n_cells; ++c) {
        m.edge_offset[c] = running;
        running += m.edge_count[c];
    }
    if (running != m.directed) throw std::logic_error("dual mesh directed edge count mismatch");

    m.area_m2.resize(n_cells);
    m.nb_cell.resize(m.directed);
    m.nb_corner.resize(m.directed);
    m.nb_edge.assign(m.directed, none);
    m.normal_east.resize(m.directed);
    m.normal_north.resize(m.directed);
    std::vector<double> length(m.directed), distance(m.directed);

    parallel_for(n_cells, [&](std::size_t c) {
        const std::uint32_t s = source_of[c];
        const std::uint32_t deg = m.edge_count[c];
        std::array<std::pair<double, std::uint32_t>, 6> order{};
        for (std::uint32_t k = 0; k < deg; ++k) {
            const std::uint32_t ci = inc.face[inc.offset[s] + k];
            const V3& p = corner[ci];
            const V3 tangent = sub(p, scale(up[c], dot(p, up[c])));
            order[k] = {std::atan2(dot(tangent, north[c]), dot(tangent, east[c])), ci};
        }
        std::sort(order.begin(), order.begin() + deg, [](const auto& a, const auto& b) {
            if (a.first == b.first) return a.second < b.second;
            return a.first < b.first;
        });
        double area = 0.0, compensation = 0.0;
        const std::uint32_t base = m.edge_offset[c];
        for (std::uint32_t k = 0; k < deg; ++k) {
            const std::uint32_t c1 = order[k].second;
            const std::uint32_t c2 = order[(k + 1) % deg].second;
            m.nb_corner[base + k] = c1;
            const double tri = triangle_area_unit(up[c], corner[c1], corner[c2]);
            const double corrected = tri - compensation;
            const double next = area + corrected;
            compensation = (next - area) - corrected;
            area = next;
            // The neighbour: the vertex the two faces share besides this cell's.
            std::uint32_t other = none;
            for (auto a : faces[c1]) {
                if (a == s) continue;
                if (std::find(faces[c2].begin(), faces[c2].end(), a) != faces[c2].end()) {
                    other = a;
                    break;
                }
            }
            if (other == none) throw std::logic_error("consecutive dual corners share no primal edge");
            const std::uint32_t nb = cell_of[other];
            if (nb == none || nb == c) throw std::logic_error("dual topology produced an invalid neighbour");
            m.nb_cell[base + k] = nb;
            length[base + k] = arc(corner[c1], corner[c2]) * radius_m;
            distance[base + k] = arc(up[c], up[nb]) * radius_m;
            const V3 out = outward_normal(up[c], corner[c1], corner[c2]);
            m.normal_east[base + k] = static_cast<float>(dot(out, east[c]));
            m.normal_north[base + k] = static_cast<float>(dot(out, north[c]));
        }
        m.area_m2[c] = area * radius_m * radius_m;
    });

    // Edge ids in order of first appearance: cell ascending, local order.
    m.edge_first.reserve(m.edges);
    m.edge_second.reserve(m.edges);
    m.edge_length_m.reserve(m.edges);
    m.edge_distance_m.reserve(m.edges);
    for (std::size_t c = 0; c < n_cells; ++c) {
        const std::uint32_t base = m.edge_offset[c];
        for (std::uint32_t k = 0; k < m.edge_count[c]; ++k) {
            const std::uint32_t nb = m.nb_cell[base + k];
            if (nb > c) {
                m.nb_edge[base + k] = static_cast<std::uint32_t>(m.edge_first.size());
                m.edge_first.push_back(static_cast<std::uint32_t>(c));
                m.edge_second.push_back(nb);
                m.edge_length_m.push_back(length[base + k]);
                m.edge_distance_m.push_back(distance[base + k]);
            } else {
                std::uint32_t found = none;
                const std::uint32_t nbase = m.edge_offset[nb];
                for (std::uint32_t j = 0; j < m.edge_count[nb]; ++j) {
                    if (m.nb_cell[nbase + j] == c) {
                        if (found != none) throw std::logic_error("dual mesh contains a non-manifold edge");
                        found = nbase + j;
                    }
                }
                if (found == none) throw std::logic_error("dual mesh contains an open boundary edge");
                const std::uint32_t id = m.nb_edge[found];
                if (m.edge_length_m[id] != length[base + k] ||
                    m.edge_distance_m[id] != distance[base + k]) {
                    throw std::logic_error("dual edge geometry is not reciprocal");
                }
                m.nb_edge[base + k] = id;
            }
        }
    }
    if (m.edge_first.size() != m.edges) throw std::logic_error("dual mesh produced unexpected edge count");
    return m;
}

TransportGraph transport_graph(const HostMesh& mesh) {
    TransportGraph g;
    g.area_m2 = mesh.area_m2;
    g.offset.resize(mesh.cells + 1);
    g.neighbour.resize(mesh.directed);
    g.weight.resize(mesh.directed);
    g.weight_sum.resize(mesh.cells);
    g.offset[0] = 0;
    for (std::size_t c = 0; c < mesh.cells; ++c) {
        const std::uint32_t base = mesh.edge_offset[c];
        double sum = 0.0;
        for (std::uint32_t k = 0; k < mesh.edge_count[c]; ++k) {
            const std::uint32_t e = mesh.nb_edge[base + k];
            g.neighbour[base + k] = mesh.nb_cell[base + k];
            g.weight[base + k] = mesh.edge_length_m[e] / mesh.edge_distance_m[e];
            sum += g.weight[base + k];
        }
        g.weight_sum[c] = sum;
        g.offset[c + 1] = base + mesh.edge_count[c];
    }
    return g;
}

}  // namespace psgb
