// Finite-volume operators and the implicit heat step's flux form, for sm_103a.
//
// K1 laplacian / diffusion_source  (sim/planet/operators/finite_volume.cpp:91-111,
//                                   sim/planet/surface/heat_transport.cpp:28-36,579-593)
// K2 gradient                       (finite_volume.cpp:55-89)
// K3 divergence                     (finite_volume.cpp:34-53)
// K13 transport step flux form      (heat_transport.cpp:734-770)
//
// One thread per cell over ELL slot-major neighbour arrays (coalesced per slot); the
// neighbour values are gathered through L2, where the reference's space-filling cell
// order keeps them close. Accumulation is FP64 in the reference's order without
// fused multiply-adds, so diffusion_source and gradient are bit-identical to the
// reference and the Laplacian differs only by using the precomputed l/d weight.
#include "common.cuh"
#include "profile.hpp"
#include "operators.hpp"

namespace psgb {
namespace {

template <typename T>
__global__ void k_laplacian(std::uint32_t n, std::uint32_t P, const std::int32_t* __restrict__ nbr,
                            const double* __restrict__ w, const double* __restrict__ area,
                            const T* __restrict__ in, T* __restrict__ out) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double own = static_cast<double>(in[c]);
    double sum = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const double wj = w[j * P + c];
        const double v = static_cast<double>(in[nbr[j * P + c]]);
        sum = dadd(sum, dmul(dsub(v, own), wj));
    }
    out[c] = static_cast<T>(__ddiv_rn(sum, area[c]));
}

// H = K * (sum_k w_k (T_k - T_c)) / A, the reference's diffusion_source.
__global__ void k_diffusion_source(std::uint32_t n, std::uint32_t P, const std::int32_t* __restrict__ nbr,
                                   const double* __restrict__ w, const double* __restrict__ area,
                                   double conductance, const double* __restrict__ t,
                                   double* __restrict__ out) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double own = t[c];
    double sum = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) sum = dadd(sum, dmul(dsub(t[nbr[j * P + c]], own), w[j * P + c]));
    out[c] = __ddiv_rn(dmul(conductance, sum), area[c]);
}

// A node's area-weighted mean of its fine cells' values, summed over the members in cell
// order and divided by the node's area (surface_energy.cpp:1285-1296); two fields at once
// (mean and slope of a response), the second optional.
__global__ void k_group_mean(std::uint32_t n, const std::uint32_t* __restrict__ member_offset,
                             const std::uint32_t* __restrict__ member, const double* __restrict__ fine_area,
                             const double* __restrict__ graph_area, const double* __restrict__ a,
                             const double* __restrict__ b, double* __restrict__ mean_a, double* __restrict__ mean_b) {
    const std::uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    double sa = 0.0, sb = 0.0;
    for (std::uint32_t k = member_offset[g]; k < member_offset[g + 1]; ++k) {
        const std::uint32_t c = member[k];
        const double area = fine_area[c];
        sa = dadd(sa, dmul(area, a[c]));
        if (b != nullptr) sb = dadd(sb, dmul(area, b[c]));
    }
    mean_a[g] = __ddiv_rn(sa, graph_area[g]);
    if (b != nullptr) mean_b[g] = __ddiv_rn(sb, graph_area[g]);
}

// Every fine cell takes its node's value (surface_energy.cpp:1583, 1595).
__global__ void k_group_scatter(std::uint32_t fine_cells, const std::uint32_t* __restrict__ group_of_cell,
                                const double* __restrict__ node_value, double* __restrict__ out) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < fine_cells) out[c] = node_value[group_of_cell[c]];
}

template <typename T>
__global__ void k_gradient(std::uint32_t n, std::uint32_t P, const std::int32_t* __restrict__ nbr,
                           const std::uint8_t* __restrict__ degree, const double* __restrict__ dist,
                           const float* __restrict__ ne, const float* __restrict__ nn,
                           const double* __restrict__ gm, const T* __restrict__ in,
                           T* __restrict__ east, T* __restrict__ north) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double own = static_cast<double>(in[c]);
    const int deg = degree[c];
    double re = 0.0, rn = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        if (j < deg) {
            const double a = static_cast<double>(ne[j * P + c]);
            const double b = static_cast<double>(nn[j * P + c]);
            const double slope = __ddiv_rn(dsub(static_cast<double>(in[nbr[j * P + c]]), own), dist[j * P + c]);
            re = dadd(re, dmul(slope, a));
            rn = dadd(rn, dmul(slope, b));
        }
    }
    const double mee = gm[c], men = gm[P + c], mnn = gm[2 * P + c], det = gm[3 * P + c];
    east[c] = static_cast<T>(__ddiv_rn(dsub(dmul(mnn, re), dmul(men, rn)), det));
    north[c] = static_cast<T>(__ddiv_rn(dsub(dmul(mee, rn), dmul(men, re)), det));
}

template <typename T>
__global__ void k_divergence(std::uint32_t n, std::uint32_t P, const std::int32_t* __restrict__ edge,
                             const std::uint8_t* __restrict__ first, const std::uint8_t* __restrict__ degree,
                             const double* __restrict__ length, const double* __restrict__ area,
                             const T* __restrict__ flux, T* __restrict__ out) {
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int deg = degree[c];
    const unsigned mask = first[c];
    double net = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        if (j < deg) {
            const int e = edge[j * P + c];
            const double f = static_cast<double>(flux[e]);
            const double signed_flux = ((mask >> j) & 1u) ? f : -f;
            net = dadd(net, dmul(signed_flux, length[e]));
        }
    }
    out[c] = static_cast<T>(__ddiv_rn(net, area[c]));
}

// ---- transport step -------------------------------------------------------------

// Right-hand side of (A/s) x + K L x = (A/s) T0 + A S, and the constant slope s = dt/C.
__global__ void k_step_rhs(std::uint32_t rows, const std::int32_t* __restrict__ tile_inst,
                           const std::int32_t* __restrict__ tile_rows, const double* __restrict__ area,
                           const double* __restrict__ slope_of, const double* __restrict__ t0,
                           const double* __restrict__ src, double* __restrict__ rhs,
                           double* __restrict__ slope, double* __restrict__ x0, unsigned long long* bytes) {
    const int tile = blockIdx.x;
    const int row = tile * kTile + threadIdx.x;
    // area, T0, S in; rhs, slope, x0 out
    if (bytes != nullptr && threadIdx.x == 0) atomicAdd(bytes, 48ull * static_cast<unsigned>(tile_rows[tile]));
    if (threadIdx.x >= tile_rows[tile]) {
        rhs[row] = 0.0;
        slope[row] = 1.0;
        x0[row] = 0.0;
        return;
    }
    const double s = slope_of[tile_inst[tile]];
    slope[row] = s;
    const double a = area[row];
    rhs[row] = dadd(dmul(__ddiv_rn(a, s), t0[row]), dmul(a, src[row]));
    x0[row] = t0[row];
}

// Flux form of the solved temperature: H = (1/A) sum_k G_k w_k (T_k - T_c), with G
// the planet's K or the per-entry conductance; T_new = T0 + s (S + H). Per-tile
// partial sums, then per-planet sums in tile order: sum A H, sum A |H|, sum A H T,
// sum A S, sum A |S|, sum A (T_new - T0) / s.
__global__ void k_step_finish(std::uint32_t P, const std::int32_t* __restrict__ tile_inst,
                              const std::int32_t* __restrict__ tile_rows,
                              const std::int32_t* __restrict__ nbr, const double* __restrict__ w,
                              const double* __restrict__ area, const double* __restrict__ conductance,
                              const double* __restrict__ edge_conductance,
                              const double* __restrict__ slope_of, const double* __restrict__ t,
                              const double* __restrict__ t0, const double* __restrict__ src,
                              double* __restrict__ h_out, double* __restrict__ t_new,
                              double* __restrict__ partial, unsigned long long* bytes) {
    const int tile = blockIdx.x;
    const int row = tile * kTile + threadIdx.x;
    const int inst = tile_inst[tile];
    // columns, weights (and per-entry conductances), area, T, T0, S in; H, T_new out
    if (bytes != nullptr && threadIdx.x == 0)
        atomicAdd(bytes, (edge_conductance != nullptr ? 168ull : 120ull) * static_cast<unsigned>(tile_rows[tile]));
    double v[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (threadIdx.x < tile_rows[tile]) {
        const double own = t[row];
        double sum = 0.0;
        double h;
        if (edge_conductance == nullptr) {
#pragma unroll
            for (int j = 0; j < 6; ++j) sum = dadd(sum, dmul(dsub(t[nbr[j * P + row]], own), w[j * P + row]));
            h = __ddiv_rn(dmul(conductance[inst], sum), area[row]);
        } else {
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                const double g = dmul(edge_conductance[j * P + row], w[j * P + row]);
                sum = dadd(sum, dmul(g, dsub(t[nbr[j * P + row]], own)));
            }
            h = __ddiv_rn(sum, area[row]);
        }
        const double s = slope_of[inst];
        const double tn = dadd(t0[row], dmul(s, dadd(src[row], h)));
        h_out[row] = h;
        t_new[row] = tn;
        const double a = area[row];
        const double flux = dmul(a, h);
        v[0] = flux;
        v[1] = fabs(flux);
        v[2] = dmul(flux, own);
        v[3] = dmul(a, src[row]);
        v[4] = fabs(v[3]);
        v[5] = dmul(a, __ddiv_rn(dsub(tn, t0[row]), s));
    }
    __shared__ double scratch[6][8];
    block_sum256<double, 6>(v, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 6; ++q) partial[tile * 8 + q] = v[q];
    }
}

// Per-planet sums of the tile partials, in tile order.
__global__ void k_sum_tiles(std::uint32_t instances, const std::uint32_t* __restrict__ tile_begin,
                            const double* __restrict__ partial, int nq, double* __restrict__ out) {
    const std::uint32_t inst = blockIdx.x;
    if (inst >= instances) return;
    const int q = threadIdx.x;
    if (q >= nq) return;
    double s = 0.0;
    for (std::uint32_t t = tile_begin[inst]; t < tile_begin[inst + 1]; ++t) s += partial[t * 8 + q];
    out[inst * 8 + q] = s;
}

__global__ void k_mask_rhs(std::size_t n, const double* __restrict__ slope, double* __restrict__ rhs) {
    const std::size_t i = blockIdx.x * std::size_t(blockDim.x) + threadIdx.x;
    if (i < n && !(slope[i] > 0.0)) rhs[i] = 0.0;
}

}  // namespace

void launch_mask_rhs(std::size_t n, const double* slope, double* rhs, cudaStream_t st) {
    PSGB_LAUNCH(kFamStep, st, k_mask_rhs<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(n, slope, rhs));
}

template <typename T>
void launch_laplacian(const DevMesh& m, const T* in, T* out, cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_laplacian<T><<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.p, m.nbr, m.w, m.area, in, out));
}
template <typename T>
void launch_gradient(const DevMesh& m, const T* in, T* east, T* north, cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_gradient<T><<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.p, m.nbr, m.degree, m.dist, m.ne, m.nn, m.gm,
                                                     in, east, north));
}
template <typename T>
void launch_divergence(const DevMesh& m, const T* flux, T* out, cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_divergence<T><<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.p, m.edge, m.first, m.degree, m.edge_length,
                                                       m.area, flux, out));
}
void launch_diffusion_source(const DevMesh& m, double conductance, const double* t, double* out,
                             cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_diffusion_source<<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.p, m.nbr, m.w, m.graph_area, conductance, t, out));
}

void launch_group_mean(const DevMesh& m, const double* a, const double* b, double* mean_a, double* mean_b,
                       cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_group_mean<<<(m.n + 255) / 256, 256, 0, st>>>(m.n, m.member_offset, m.member, m.fine_area,
                                                                               m.graph_area, a, b, mean_a, mean_b));
}
void launch_group_scatter(const DevMesh& m, const double* node_value, double* out, cudaStream_t st) {
    PSGB_LAUNCH(kFamOperator, st, k_group_scatter<<<(m.fine_cells + 255) / 256, 256, 0, st>>>(m.fine_cells, m.group_of_cell,
                                                                                           node_value, out));
}

template void launch_laplacian<float>(const DevMesh&, const float*, float*, cudaStream_t);
template void launch_laplacian<double>(const DevMesh&, const double*, double*, cudaStream_t);
template void launch_gradient<float>(const DevMesh&, const float*, float*, float*, cudaStream_t);
template void launch_gradient<double>(const DevMesh&, const double*, double*, double*, cudaStream_t);
template void launch_divergence<float>(const DevMesh&, const float*, float*, cudaStream_t);
template void launch_divergence<double>(const DevMesh&, const double*, double*, cudaStream_t);

void launch_step_rhs(const StepView& v, const double* t0, const double* src, double* rhs, double* slope,
                     double* x0, cudaStream_t st) {
    PSGB_LAUNCH(kFamStep, st, k_step_rhs<<<v.tiles, kTile, 0, st>>>(v.rows, v.tile_inst, v.tile_rows, v.area, v.slope_of, t0, src,
                                          rhs, slope, x0, v.bytes));
}

void launch_step_finish(const StepView& v, const double* t, const double* t0, const double* src,
                        double* h, double* t_new, double* partial, double* sums, cudaStream_t st) {
    PSGB_LAUNCH(kFamStep, st, k_step_finish<<<v.tiles, kTile, 0, st>>>(v.rows, v.tile_inst, v.tile_rows, v.nbr, v.w, v.area,
                                             v.conductance, v.edge_conductance, v.slope_of, t, t0, src, h,
                                             t_new, partial, v.bytes));
    PSGB_LAUNCH(kFamStep, st, k_sum_tiles<<<v.instances, 32, 0, st>>>(v.instances, v.tile_begin, partial, 6, sums));
}

}  // namespace psgb
