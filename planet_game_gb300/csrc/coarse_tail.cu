// The coarse tail of the V-cycle (see coarse_tail.hpp): one block of four 256-thread tile
// groups per planet. The block walks its planet's tiles of each level (group g takes
// tiles g, g + 4, ...), calls the shared per-tile phases, and meets at a block barrier
// between phases; the dense coarsest solve uses the block's 32 warps, one row each.
#define PSGB_PHASE_RESTRICT
#include "coarse_tail.hpp"
#include "phases.cuh"
#include "profile.hpp"

#include <type_traits>

namespace psgb {
namespace {

template <typename F>
__device__ __forceinline__ void tail_widths(unsigned width, F&& f) {
    switch (width) {
        case 6: f(std::integral_constant<int, 6>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 12: f(std::integral_constant<int, 12>{}); break;
        default: f(std::integral_constant<int, 16>{}); break;
    }
}

template <typename T>
struct TailPair {
    T* first;
    T* second;
};

template <typename T>
__device__ __forceinline__ TailPair<T> tail_pair(const TailArgs<T>& a, int l) {
    T* X = a.level[l].x;
    T* Y = a.level[l].y;
    return a.starts_in_x[l] ? TailPair<T>{X, Y} : TailPair<T>{Y, X};
}

// The planet's tiles of level l, split over the block's four groups.
#define PSGB_PLANET_TILES(a, l, inst, gid)                                                      \
    for (int tile = static_cast<int>((a).tile_range[((l) * (a).instances + (inst)) * 2]) + (gid), \
             tile_end = static_cast<int>((a).tile_range[((l) * (a).instances + (inst)) * 2] +    \
                                         (a).tile_range[((l) * (a).instances + (inst)) * 2 + 1]); \
         tile < tile_end; tile += ph::kGroups)

template <typename T>
__global__ void __launch_bounds__(1024, 1) k_coarse_tail(const __grid_constant__ TailArgs<T> a) {
    pdl_begin();
    const int inst = static_cast<int>(blockIdx.x);
    const int gid = static_cast<int>(threadIdx.x >> 8), lane = static_cast<int>(threadIdx.x & 255);
    const int coarsest = a.dense.level[inst];
    if (coarsest < a.first || !ph::gate_open(a.sc, inst, a.gate)) return;
    const T omega = a.omega;
    // Down: the level's remaining pre-sweeps (its first sweep came with the restriction
    // into it), residual, restriction fused with the next level's first sweep.
    for (int l = a.first; l < coarsest; ++l) {
        const PersistentLevel<T>& L = a.level[l];
        const LevelView<T>& lv = L.view;
        TailPair<T> p = tail_pair(a, l);
        for (int k = 1; k < a.pre[l]; ++k) {
            tail_widths(lv.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    PSGB_PLANET_TILES(a, l, inst, gid)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, gid, lane, L.b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, a.gate);
                } else {
                    PSGB_PLANET_TILES(a, l, inst, gid)
                        ph::smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, p.second, omega, a.sc, a.gate);
                }
            });
            __syncthreads();
            T* t = p.first; p.first = p.second; p.second = t;
        }
        tail_widths(lv.width, [&](auto W) {
            PSGB_PLANET_TILES(a, l, inst, gid)
                ph::residual<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, L.r, a.sc, a.gate);
        });
        __syncthreads();
        const PersistentLevel<T>& C = a.level[l + 1];
        const TailPair<T> pc = tail_pair(a, l + 1);
        PSGB_PLANET_TILES(a, l + 1, inst, gid)
            ph::restrict_zero<T, 1>(C.view, tile, lane, L.member_offset, L.member, L.r, C.b, pc.first, omega, a.sc, a.gate);
        __syncthreads();
    }
    // The planet's coarsest level: x = A^-1 b, one warp per row.
    {
        const int n = static_cast<int>(a.dense.size[inst]);
        const PersistentLevel<T>& L = a.level[coarsest];
        for (int row = static_cast<int>(threadIdx.x >> 5); row < n; row += 32)
            ph::dense_row<T>(a.dense, inst, row, static_cast<int>(threadIdx.x & 31), a.dense_inv, L.b, L.x);
        __syncthreads();
    }
    // Up: prolongation fused with the first post-sweep, then the remaining post-sweeps.
    for (int l = coarsest - 1; l >= a.first; --l) {
        const PersistentLevel<T>& L = a.level[l];
        const LevelView<T>& lv = L.view;
        const T* e = a.level[l + 1].x;
        TailPair<T> p = tail_pair(a, l);
        if ((a.pre[l] - 1) & 1) { T* t = p.first; p.first = p.second; p.second = t; }   // where the down sweeps ended
        if (a.post[l] == 0) {
            PSGB_PLANET_TILES(a, l, inst, gid) ph::prolong<T, 1>(lv, tile, lane, L.agg, e, p.first, a.sc, a.gate);
            __syncthreads();
            continue;
        }
        tail_widths(lv.width, [&](auto W) {
            PSGB_PLANET_TILES(a, l, inst, gid)
                ph::prolong_smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.agg, e, L.b, p.first, p.second, omega, a.sc,
                                                             a.gate);
        });
        __syncthreads();
        { T* t = p.first; p.first = p.second; p.second = t; }
        for (int k = 1; k < a.post[l]; ++k) {
            tail_widths(lv.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    PSGB_PLANET_TILES(a, l, inst, gid)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, gid, lane, L.b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, a.gate);
                } else {
                    PSGB_PLANET_TILES(a, l, inst, gid)
                        ph::smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, p.second, omega, a.sc, a.gate);
                }
            });
            __syncthreads();
            T* t = p.first; p.first = p.second; p.second = t;
        }
    }
}

}  // namespace

template <typename T>
void launch_coarse_tail(const TailArgs<T>& args, cudaStream_t st) {
    PSGB_LAUNCH(kFamSmoothCoarse, st, launch_pdl(k_coarse_tail<T>, args.instances, 1024, st, args));
}

template void launch_coarse_tail<float>(const TailArgs<float>&, cudaStream_t);
template void launch_coarse_tail<double>(const TailArgs<double>&, cudaStream_t);

}  // namespace psgb
