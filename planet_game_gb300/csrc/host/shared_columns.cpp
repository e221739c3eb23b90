// The fine level's columns once per distinct graph of a batch (see shared_columns.hpp).
#include "shared_columns.hpp"

namespace psgb {

SharedColumns shared_columns(const std::vector<const HostLevel*>& fine, const std::vector<std::int64_t>& base,
                             const std::vector<std::int32_t>& tile_inst, std::size_t width) {
    SharedColumns out;
    const std::size_t planets = fine.size();
    std::vector<int> graph_of(planets, -1);
    std::vector<std::size_t> holder;   // a planet holding each distinct graph
    for (std::size_t i = 0; i < planets; ++i) {
        if (base[i] < 0) continue;
        const HostLevel& h = *fine[i];
        for (std::size_t g = 0; g < holder.size() && graph_of[i] < 0; ++g) {
            const HostLevel& o = *fine[holder[g]];
            if (h.size == o.size && h.offset == o.offset && h.column == o.column) graph_of[i] = static_cast<int>(g);
        }
        if (graph_of[i] < 0) {
            graph_of[i] = static_cast<int>(holder.size());
            holder.push_back(i);
        }
    }
    std::size_t present = 0;
    for (std::size_t i = 0; i < planets; ++i) present += base[i] >= 0 ? 1 : 0;
    if (holder.size() == present) return out;
    std::vector<std::uint32_t> start(holder.size());
    std::uint32_t pitch = 0;
    for (std::size_t g = 0; g < holder.size(); ++g) {
        start[g] = pitch;
        pitch += pad_rows(fine[holder[g]]->size);
    }
    out.pitch = pitch;
    out.scol.assign(width * pitch, 0);
    for (std::size_t g = 0; g < holder.size(); ++g) {
        const HostLevel& h = *fine[holder[g]];
        for (std::uint32_t r = 0; r < pad_rows(h.size); ++r)
            for (std::size_t j = 0; j < width; ++j) out.scol[j * pitch + start[g] + r] = static_cast<std::int32_t>(r);
        for (std::uint32_t r = 0; r < h.size; ++r)
            for (std::uint32_t k = h.offset[r]; k < h.offset[r + 1]; ++k)
                out.scol[(k - h.offset[r]) * pitch + start[g] + r] = static_cast<std::int32_t>(h.column[k]);
    }
    out.shift.assign(2 * tile_inst.size(), 0);
    for (std::size_t t = 0; t < tile_inst.size(); ++t) {
        const int i = tile_inst[t];
        const auto first = static_cast<std::int32_t>(base[i]);
        out.shift[2 * t] = first;
        out.shift[2 * t + 1] = first - static_cast<std::int32_t>(start[graph_of[i]]);
    }
    return out;
}

}  // namespace psgb
