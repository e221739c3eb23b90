// CPU ORACLE - test infrastructure only (tests/, smoke() and bench.py's CPU legs).
//
// A plain, single-threaded restatement of the reference's mesh builder, make_icosphere
// (sim/planet/mesh/icosphere.cpp:200-419), with its helpers (:55-139: spherical triangle
// area, great-circle angle, outward edge normal, circumcentre, Lloyd relaxation, the
// icosahedron), the local tangent basis (sim/planet/coordinates/local_tangent_basis.cpp:8-24)
// and the transport graph of that mesh (sim/planet/surface/heat_transport.cpp:433-452).
// It lets the CPU legs of the benchmark build their planets without the product library.
// Every step keeps the reference's FP64 operation order, so the arrays are the
// reference's bit for bit (pinned by tests/test_oracle_mesh.py against the same SHA-256
// digests as the product's builder).
//
// The relaxed unit-sphere mesh is the same for every radius; it is kept per level and a
// radius only scales the arc lengths (angle * R) and areas (area * R * R), as the
// reference forms them.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <vector>

namespace {

struct P3 {
    double x = 0.0, y = 0.0, z = 0.0;
};
P3 operator+(const P3& a, const P3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
P3 operator-(const P3& a, const P3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
P3 operator*(const P3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dot(const P3& a, const P3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
P3 cross(const P3& a, const P3& b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
P3 unit(const P3& a) {
    const double m = std::sqrt(dot(a, a));
    if (!(m > 0.0) || !std::isfinite(m)) throw std::invalid_argument("oracle mesh: zero vector");
    return {a.x / m, a.y / m, a.z / m};
}

// 2 atan2(|a . (b x c)|, 1 + a.b + b.c + c.a)  (icosphere.cpp:55-60)
double triangle_area(const P3& a, const P3& b, const P3& c) {
    const double num = std::abs(dot(a, cross(b, c)));
    const double den = 1.0 + dot(a, b) + dot(b, c) + dot(c, a);
    return 2.0 * std::atan2(num, den);
}

double arc(const P3& a, const P3& b) { return std::acos(std::clamp(dot(a, b), -1.0, 1.0)); }

P3 circumcentre(const P3& a, const P3& b, const P3& c) {
    P3 n = unit(cross(b - a, c - a));
    if (dot(n, a + b + c) < 0.0) n = n * -1.0;
    return n;
}

P3 outward_normal(const P3& centre, const P3& c1, const P3& c2) {
    P3 n = unit(cross(c1, c2));
    if (dot(n, centre) > 0.0) n = n * -1.0;
    return unit(n - centre * dot(n, centre));
}

using Tri = std::array<std::uint32_t, 3>;

void lloyd(std::vector<P3>& v, const std::vector<Tri>& faces, int sweeps) {
    std::vector<P3> acc(v.size());
    for (int it = 0; it < sweeps; ++it) {
        std::fill(acc.begin(), acc.end(), P3{});
        for (const Tri& f : faces) {
            const P3 cc = circumcentre(v[f[0]], v[f[1]], v[f[2]]);
            for (int k = 0; k < 3; ++k) {
                const P3& g = v[f[k]];
                const P3* side[2] = {&v[f[(k + 1) % 3]], &v[f[(k + 2) % 3]]};
                for (const P3* s : side) {
                    const P3 mid = unit(g + *s);
                    const double area = triangle_area(g, mid, cc);
                    acc[f[k]] = acc[f[k]] + unit(g + mid + cc) * area;
                }
            }
        }
        for (std::size_t i = 0; i < v.size(); ++i) v[i] = unit(acc[i]);
    }
}

// The unit-sphere mesh of one level: everything but the radius.
struct UnitMesh {
    std::uint32_t cells = 0, edges = 0, corners = 0;
    std::vector<P3> centre, east, north, corner_unit;
    std::vector<std::uint32_t> source_vertex, edge_offset, neighbor, edge, corner, edge_first, edge_second;
    std::vector<std::uint8_t> edge_count;
    std::vector<float> normal_east, normal_north;
    std::vector<double> area_unit, edge_arc, centre_arc;
};

std::unique_ptr<UnitMesh> build_unit(std::uint32_t level) {
    const double phi = 1.6180339887498948482;
    std::vector<P3> v = {{-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0}, {0, -1, phi}, {0, 1, phi},
                         {0, -1, -phi}, {0, 1, -phi}, {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}};
    for (P3& p : v) p = unit(p);
    std::vector<Tri> faces = {{0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11},
                              {1, 5, 9},  {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                              {3, 9, 4},  {3, 4, 2},  {3, 2, 6},   {3, 6, 8},  {3, 8, 9},
                              {4, 9, 5},  {2, 4, 11}, {6, 2, 10},  {8, 6, 7},  {9, 8, 1}};
    for (std::uint32_t l = 0; l < level; ++l) {
        std::map<std::uint64_t, std::uint32_t> mids;
        auto mid = [&](std::uint32_t a, std::uint32_t b) {
            const std::uint64_t key = (std::uint64_t(std::min(a, b)) << 32) | std::max(a, b);
            auto it = mids.find(key);
            if (it != mids.end()) return it->second;
            const auto id = static_cast<std::uint32_t>(v.size());
            v.push_back(unit(v[a] + v[b]));
            mids.emplace(key, id);
            return id;
        };
        std::vector<Tri> next;
        next.reserve(4 * faces.size());
        for (const Tri& f : faces) {
            const std::uint32_t a = mid(f[0], f[1]), b = mid(f[1], f[2]), c = mid(f[2], f[0]);
            next.push_back({f[0], a, c});
            next.push_back({f[1], b, a});
            next.push_back({f[2], c, b});
            next.push_back({a, b, c});
        }
        faces.swap(next);
        lloyd(v, faces, 20);
    }
    auto m = std::make_unique<UnitMesh>();
    m->cells = static_cast<std::uint32_t>(v.size());
    m->corners = static_cast<std::uint32_t>(faces.size());
    // cells in the order their vertices first appear in the face list
    std::vector<std::int64_t> cell_of(v.size(), -1);
    for (const Tri& f : faces)
        for (std::uint32_t s : f)
            if (cell_of[s] < 0) {
                cell_of[s] = static_cast<std::int64_t>(m->source_vertex.size());
                m->source_vertex.push_back(s);
            }
    std::vector<std::vector<std::uint32_t>> touching(v.size());
    for (std::size_t k = 0; k < faces.size(); ++k) {
        const Tri& f = faces[k];
        m->corner_unit.push_back(circumcentre(v[f[0]], v[f[1]], v[f[2]]));
        for (std::uint32_t s : f) touching[s].push_back(static_cast<std::uint32_t>(k));
    }
    for (std::uint32_t c = 0; c < m->cells; ++c) {
        const P3 up = unit(v[m->source_vertex[c]]);
        const double h = std::hypot(up.x, up.y);
        const P3 east = h > 1.0e-12 ? P3{-up.y / h, up.x / h, 0.0} : P3{0.0, 1.0, 0.0};
        m->centre.push_back(up);
        m->east.push_back(east);
        m->north.push_back(unit(cross(up, east)));
    }
    std::map<std::uint64_t, std::uint32_t> edge_id;
    for (std::uint32_t c = 0; c < m->cells; ++c) {
        const P3& up = m->centre[c];
        const std::uint32_t src = m->source_vertex[c];
        struct Around {
            std::uint32_t corner;
            double angle;
        };
        std::vector<Around> ring;
        for (std::uint32_t k : touching[src]) {
            const P3& q = m->corner_unit[k];
            const P3 t = q - up * dot(q, up);
            ring.push_back({k, std::atan2(dot(t, m->north[c]), dot(t, m->east[c]))});
        }
        if (ring.size() != 5 && ring.size() != 6) throw std::logic_error("oracle mesh: cell of neither 5 nor 6 sides");
        std::sort(ring.begin(), ring.end(), [](const Around& a, const Around& b) {
            return a.angle == b.angle ? a.corner < b.corner : a.angle < b.angle;
        });
        m->edge_offset.push_back(static_cast<std::uint32_t>(m->neighbor.size()));
        m->edge_count.push_back(static_cast<std::uint8_t>(ring.size()));
        double area = 0.0, carry = 0.0;   // Kahan sum of the cell's triangles
        for (std::size_t k = 0; k < ring.size(); ++k) {
            const std::uint32_t k1 = ring[k].corner, k2 = ring[(k + 1) % ring.size()].corner;
            m->corner.push_back(k1);
            const double tri = triangle_area(up, m->corner_unit[k1], m->corner_unit[k2]) - carry;
            const double sum = area + tri;
            carry = (sum - area) - tri;
            area = sum;
            // the neighbour: the vertex the two faces share besides this cell's own
            std::int64_t other = -1;
            for (std::uint32_t s : faces[k1]) {
                if (s == src) continue;
                if (std::find(faces[k2].begin(), faces[k2].end(), s) != faces[k2].end()) {
                    other = s;
                    break;
                }
            }
            if (other < 0) throw std::logic_error("oracle mesh: corners share no edge");
            const auto nb = static_cast<std::uint32_t>(cell_of[static_cast<std::size_t>(other)]);
            const std::uint64_t key = (std::uint64_t(std::min(c, nb)) << 32) | std::max(c, nb);
            auto found = edge_id.find(key);
            if (found == edge_id.end()) {
                found = edge_id.emplace(key, static_cast<std::uint32_t>(m->edge_first.size())).first;
                m->edge_first.push_back(std::min(c, nb));
                m->edge_second.push_back(std::max(c, nb));
                m->edge_arc.push_back(arc(m->corner_unit[k1], m->corner_unit[k2]));
                m->centre_arc.push_back(arc(up, m->centre[nb]));
            }
            const P3 out = outward_normal(up, m->corner_unit[k1], m->corner_unit[k2]);
            m->neighbor.push_back(nb);
            m->edge.push_back(found->second);
            m->normal_east.push_back(static_cast<float>(dot(out, m->east[c])));
            m->normal_north.push_back(static_cast<float>(dot(out, m->north[c])));
        }
        m->area_unit.push_back(area);
    }
    m->edges = static_cast<std::uint32_t>(m->edge_first.size());
    return m;
}

std::mutex g_mutex;
std::map<std::uint32_t, std::unique_ptr<UnitMesh>> g_levels;

const UnitMesh& unit_mesh(std::uint32_t level) {
    if (level > 10) throw std::invalid_argument("oracle mesh: level above 10");
    std::lock_guard<std::mutex> lock(g_mutex);
    auto& slot = g_levels[level];
    if (!slot) slot = build_unit(level);
    return *slot;
}

void put3(const std::vector<P3>& v, double* out) {
    for (std::size_t i = 0; i < v.size(); ++i) {
        out[3 * i] = v[i].x;
        out[3 * i + 1] = v[i].y;
        out[3 * i + 2] = v[i].z;
    }
}

}  // namespace

extern "C" {

// Cells, undirected edges, corners of the level-`level` mesh; 0 on success.
int orc_icosphere_counts(std::uint32_t level, std::uint64_t* cells, std::uint64_t* edges, std::uint64_t* corners) {
    try {
        const UnitMesh& m = unit_mesh(level);
        *cells = m.cells;
        *edges = m.edges;
        *corners = m.corners;
        return 0;
    } catch (...) {
        return 1;
    }
}

// The reference PlanetMesh's arrays at `radius_m` (sizes from orc_icosphere_counts: n
// cells, e edges, k corners, d = 2e directed entries) and the transport graph's
// weights l/d per directed entry and their per-cell sums.
int orc_icosphere(std::uint32_t level, double radius_m, double* center, double* east, double* north, double* area_m2,
                  std::uint32_t* source_vertex, std::uint32_t* edge_offset, std::uint8_t* edge_count,
                  std::uint32_t* neighbor, std::uint32_t* edge, std::uint32_t* corner, float* normal_east,
                  float* normal_north, std::uint32_t* edge_first, std::uint32_t* edge_second, double* edge_length_m,
                  double* edge_distance_m, double* corner_unit, double* graph_weight, double* graph_weight_sum) {
    try {
        if (!(radius_m > 0.0) || !std::isfinite(radius_m)) return 2;
        const UnitMesh& m = unit_mesh(level);
        put3(m.centre, center);
        put3(m.east, east);
        put3(m.north, north);
        put3(m.corner_unit, corner_unit);
        std::memcpy(source_vertex, m.source_vertex.data(), m.cells * sizeof(std::uint32_t));
        std::memcpy(edge_offset, m.edge_offset.data(), m.cells * sizeof(std::uint32_t));
        std::memcpy(edge_count, m.edge_count.data(), m.cells);
        const std::size_t d = m.neighbor.size();
        std::memcpy(neighbor, m.neighbor.data(), d * sizeof(std::uint32_t));
        std::memcpy(edge, m.edge.data(), d * sizeof(std::uint32_t));
        std::memcpy(corner, m.corner.data(), d * sizeof(std::uint32_t));
        std::memcpy(normal_east, m.normal_east.data(), d * sizeof(float));
        std::memcpy(normal_north, m.normal_north.data(), d * sizeof(float));
        std::memcpy(edge_first, m.edge_first.data(), m.edges * sizeof(std::uint32_t));
        std::memcpy(edge_second, m.edge_second.data(), m.edges * sizeof(std::uint32_t));
        for (std::uint32_t e = 0; e < m.edges; ++e) {
            edge_length_m[e] = m.edge_arc[e] * radius_m;
            edge_distance_m[e] = m.centre_arc[e] * radius_m;
        }
        for (std::uint32_t c = 0; c < m.cells; ++c) {
            area_m2[c] = m.area_unit[c] * radius_m * radius_m;
            double sum = 0.0;
            for (std::uint32_t k = m.edge_offset[c]; k < m.edge_offset[c] + m.edge_count[c]; ++k) {
                const std::uint32_t e = m.edge[k];
                graph_weight[k] = edge_length_m[e] / edge_distance_m[e];
                sum += graph_weight[k];
            }
            graph_weight_sum[c] = sum;
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

}  // extern "C"

// ---- the sub-step-mean insolation of the benchmark's source term -----------------------
//
// compute_substep_mean_insolation (sim/planet/orbit/substep_forcing.cpp:102-127) with
// daily_mean_insolation_W_m2 (:35-56): per cell, the weighted sum over the sub-step's 16
// orbit nodes of the daily-mean insolation at the cell's latitude (sin = z, cos =
// sqrt(x^2 + y^2) of its unit centre), stored in FP32. The nodes (weight, sin and cos of
// the declination, incident flux) are the reference's own for the sub-step, passed in.
namespace {

double daily_mean(double sin_lat, double cos_lat, double sin_dec, double cos_dec, double flux) {
    const double pi = 3.14159265358979323846;
    const double a = sin_lat * sin_dec;
    const double b = cos_lat * cos_dec;
    double h = 0.0;
    if (b <= 0.0) {
        h = a > 0.0 ? pi : 0.0;
    } else {
        const double c = -a / b;
        if (c <= -1.0) {
            h = pi;
        } else if (c < 1.0) {
            h = std::acos(c);
        }
    }
    const double value = flux / pi * (h * a + b * std::sin(h));
    return std::max(0.0, value);
}

}  // namespace

extern "C" void orc_substep_mean_insolation(std::uint64_t cells, const double* center, const double* weight,
                                            const double* sin_dec, const double* cos_dec, const double* flux,
                                            std::uint32_t nodes, float* out) {
    for (std::uint64_t c = 0; c < cells; ++c) {
        const double x = center[3 * c], y = center[3 * c + 1], z = center[3 * c + 2];
        const double sin_lat = z;
        const double cos_lat = std::sqrt(x * x + y * y);
        double mean = 0.0;
        for (std::uint32_t k = 0; k < nodes; ++k) {
            mean += weight[k] * daily_mean(sin_lat, cos_lat, sin_dec[k], cos_dec[k], flux[k]);
        }
        out[c] = static_cast<float>(mean);
    }
}
