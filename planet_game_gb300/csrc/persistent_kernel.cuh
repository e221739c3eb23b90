// Device side of the persistent cooperative solver (persistent.cu has the host side):
// included by one translation unit per precision (persistent_f32.cu, persistent_f64.cu),
// which instantiate the two entry points below for their type and compile side by side.
// The whole solve is one kernel per type, so one type per translation unit halves the
// build's longest compile.
#pragma once

#define PSGB_PHASE_RESTRICT
#include "persistent.hpp"
#include "phases.cuh"
#include "profile.hpp"
#include "solver.hpp"

#include <type_traits>

namespace psgb {
namespace {

// A barrier normally completes in microseconds. A wait gives up after kBarrierTimeoutNs of
// device time (or kSpinLimit polls, whichever comes first): it then records the error and
// the kernel returns.
constexpr unsigned long long kBarrierTimeoutNs = 5000000000ull;
constexpr unsigned kSpinLimit = 1u << 28;

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
    return *reinterpret_cast<const volatile unsigned*>(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier. Thread 0 of each block: release fence, arrive; the last block to arrive
// resets the count and advances the generation; the others poll the generation (bounded).
// Returns false when the kernel must stop (a wait ran out here or in another block).
__device__ bool grid_barrier(const PersistentSync& sync) {
    __shared__ int stop;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_volatile(sync.gen);
        __threadfence();
        const unsigned arrived = atomicAdd(sync.count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(sync.count, 0u);
            __threadfence();
            atomicAdd(sync.gen, 1u);
        } else {
            const unsigned long long start = global_ns();
            unsigned spins = 0;
            while (ld_volatile(sync.gen) == gen) {
                if (ld_volatile(sync.error) != 0u) break;
                ++spins;
                if (spins > kSpinLimit || ((spins & 1023u) == 0u && global_ns() - start > kBarrierTimeoutNs)) {
                    atomicExch(sync.error, 1u);
                    break;
                }
                if (spins > 4096u) __nanosleep(64);
            }
        }
        __threadfence();
        stop = ld_volatile(sync.error) != 0u;
    }
    __syncthreads();
    return stop == 0;
}

// Every block reads the same scalars after the same barrier, so every block decides alike.
__device__ bool any_outer_running(const InstanceScalars* sc, unsigned instances) {
    for (unsigned i = 0; i < instances; ++i) {
        if (*reinterpret_cast<const volatile int*>(&sc[i].outer_status) == kRunning) return true;
    }
    return false;
}

__device__ bool any_inner_running(const InstanceScalars* sc, unsigned instances) {
    for (unsigned i = 0; i < instances; ++i) {
        const int outer = *reinterpret_cast<const volatile int*>(&sc[i].outer_status);
        const int inner = *reinterpret_cast<const volatile int*>(&sc[i].status);
        if (outer == kRunning && inner == kRunning) return true;
    }
    return false;
}

// This thread's tile group: groups 0..3 of the block, lane 0..255 within the group.
struct Group {
    int gid, lane, first, stride;
};

__device__ __forceinline__ Group group_of() {
    const int gid = static_cast<int>(threadIdx.x >> 8);
    return Group{gid, static_cast<int>(threadIdx.x & 255), static_cast<int>(blockIdx.x) * ph::kGroups + gid,
                 static_cast<int>(gridDim.x) * ph::kGroups};
}

// Tiles per tile set of every phase here (rows per thread).
constexpr int kPR = 2;

#define PSGB_SETS(lv, G) \
    for (int t0 = (G).first * kPR; t0 < static_cast<int>((lv).tiles); t0 += (G).stride * kPR)
#define PSGB_BARRIER(a) \
    if (!grid_barrier((a).sync)) return false

// f(std::integral_constant<int, W>) for the level's ELL width.
template <typename F>
__device__ __forceinline__ void with_width(unsigned width, F&& f) {
    switch (width) {
        case 6: f(std::integral_constant<int, 6>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 12: f(std::integral_constant<int, 12>{}); break;
        default: f(std::integral_constant<int, 16>{}); break;
    }
}

template <typename T>
using Args = PersistentArgs<T>;

// Coarsest-level solves of the planets whose coarsest level is `level`: one warp per row,
// the rows of the level's dense blocks spread over all warps of the grid.
template <typename T>
__device__ void dense_phase(const Args<T>& a, int level, const T* b, T* x, int gate) {
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned warps = (gridDim.x * blockDim.x) >> 5;
    const unsigned begin = a.dense_block_offset[level], rows = (a.dense_block_offset[level + 1] - begin) * 8u;
    for (unsigned k = warp; k < rows; k += warps) {
        const int2 blk = a.dense_blocks[begin + k / 8u];
        const int row = blk.y + static_cast<int>(k % 8u);
        if (row >= static_cast<int>(a.dense.size[blk.x]) || !ph::gate_open(a.sc, blk.x, gate)) continue;
        ph::dense_row<T>(a.dense, blk.x, row, static_cast<int>(threadIdx.x & 31), a.dense_inv, b, x);
    }
}

// The two buffers of level l: the first (zero-start) sweep writes `first`.
template <typename T>
struct Pair {
    T* first;
    T* second;
};

template <typename T>
__device__ __forceinline__ Pair<T> pair_of(const Args<T>& a, int l, T* x) {
    T* X = l == 0 ? x : a.level[l].x;
    T* Y = a.level[l].y;
    return a.starts_in_x[l] ? Pair<T>{X, Y} : Pair<T>{Y, X};
}

// x = M^-1 rhs for every planet the gate admits. The fine level's zero-start sweep has
// already been written by the Krylov phase before (fused there), as in the kernel path.
template <typename T>
__device__ bool vcycle(const Args<T>& a, const T* rhs, T* x, int gate) {
    const Group G = group_of();
    const T omega = a.omega;
    if (a.dense_at[0]) {
        dense_phase<T>(a, 0, rhs, x, gate);
        PSGB_BARRIER(a);
    }
    // Down: pre-smoothing, residual, restriction fused with the next level's first sweep.
    for (int l = 0; l + 1 < a.depth; ++l) {
        const PersistentLevel<T>& L = a.level[l];
        const LevelView<T>& lv = L.view;
        const T* b = l == 0 ? rhs : L.b;
        Pair<T> p = pair_of(a, l, x);
        // Planets whose coarsest level is this one (l >= 1) solve it in the level's first
        // phase: they do not smooth here, the others do not need them yet.
        bool dense = l > 0 && a.dense_at[l];
        for (int k = 1; k < a.pre[l]; ++k) {
            if (dense) dense_phase<T>(a, l, L.b, L.x, gate);
            dense = false;
            with_width(lv.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    for (int tile = G.first; tile < static_cast<int>(lv.tiles); tile += G.stride)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, G.gid, G.lane, b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, gate);
                } else {
                    PSGB_SETS(lv, G) ph::smooth<T, decltype(W)::value, kPR>(lv, t0, G.lane, b, p.first, p.second, omega, a.sc, gate);
                }
            });
            PSGB_BARRIER(a);
            T* t = p.first; p.first = p.second; p.second = t;
        }
        if (dense) dense_phase<T>(a, l, L.b, L.x, gate);
        with_width(lv.width, [&](auto W) {
            PSGB_SETS(lv, G) ph::residual<T, decltype(W)::value, kPR>(lv, t0, G.lane, b, p.first, L.r, a.sc, gate);
        });
        PSGB_BARRIER(a);
        const PersistentLevel<T>& C = a.level[l + 1];
        const Pair<T> pc = pair_of(a, l + 1, x);
        PSGB_SETS(C.view, G) ph::restrict_zero<T, kPR>(C.view, t0, G.lane, L.member_offset, L.member, L.r, C.b, pc.first, omega, a.sc, gate);
        PSGB_BARRIER(a);
        if (l + 2 == a.depth && a.dense_at[l + 1]) {
            dense_phase<T>(a, l + 1, C.b, C.x, gate);
            PSGB_BARRIER(a);
        }
    }
    // Up: prolongation fused with the first post-smoothing sweep.
    for (int l = a.depth - 2; l >= 0; --l) {
        const PersistentLevel<T>& L = a.level[l];
        const LevelView<T>& lv = L.view;
        const T* b = l == 0 ? rhs : L.b;
        const T* e = a.level[l + 1].x;
        Pair<T> p = pair_of(a, l, x);
        if ((a.pre[l] - 1) & 1) { T* t = p.first; p.first = p.second; p.second = t; }   // where the down sweeps ended
        if (a.post[l] == 0) {
            PSGB_SETS(lv, G) ph::prolong<T, kPR>(lv, t0, G.lane, L.agg, e, p.first, a.sc, gate);
            PSGB_BARRIER(a);
            continue;
        }
        with_width(lv.width, [&](auto W) {
            PSGB_SETS(lv, G) ph::prolong_smooth<T, decltype(W)::value, kPR>(lv, t0, G.lane, L.agg, e, b, p.first, p.second, omega, a.sc, gate);
        });
        PSGB_BARRIER(a);
        { T* t = p.first; p.first = p.second; p.second = t; }
        for (int k = 1; k < a.post[l]; ++k) {
            with_width(lv.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    for (int tile = G.first; tile < static_cast<int>(lv.tiles); tile += G.stride)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, G.gid, G.lane, b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, gate);
                } else {
                    PSGB_SETS(lv, G) ph::smooth<T, decltype(W)::value, kPR>(lv, t0, G.lane, b, p.first, p.second, omega, a.sc, gate);
                }
            });
            PSGB_BARRIER(a);
            T* t = p.first; p.first = p.second; p.second = t;
        }
    }
    return true;
}

template <typename T>
__device__ bool bicgstab(const Args<T>& a) {
    const Group G = group_of();
    const LevelView<T>& lv = a.level[0].view;
    const ReduceCtx& ctx = a.ctx;
    T *r = a.k[0], *shadow = a.k[1], *p = a.k[2], *v = a.k[3], *phat = a.k[4], *s = a.k[5], *shat = a.k[6],
      *t = a.k[7];
    const T* rhs = a.k[8];
    T* x = a.k[9];
    const T omega_j = a.omega;
    PSGB_SETS(lv, G) ph::bicg_init<T, kPR>(lv, t0, G.gid, G.lane, rhs, x, r, shadow, p, v, ctx, a.inner_tolerance, a.max_iterations);
    PSGB_BARRIER(a);
    T* phat_first = pair_of(a, 0, phat).first;
    T* shat_first = pair_of(a, 0, shat).first;
    for (int it = 0; it < a.max_iterations; ++it) {
        if (!any_inner_running(a.sc, a.instances)) break;
        PSGB_SETS(lv, G) ph::bicg_p<T, kPR>(lv, t0, G.lane, r, v, p, phat_first, omega_j, a.sc);
        PSGB_BARRIER(a);
        if (!vcycle<T>(a, p, phat, kGateRunning)) return false;
        with_width(lv.width, [&](auto W) {
            PSGB_SETS(lv, G) ph::bicg_v<T, decltype(W)::value, kPR>(lv, t0, G.gid, G.lane, phat, v, shadow, ctx);
        });
        PSGB_BARRIER(a);
        PSGB_SETS(lv, G) ph::bicg_s<T, kPR>(lv, t0, G.gid, G.lane, r, v, s, shat_first, omega_j, ctx);
        PSGB_BARRIER(a);
        if (!vcycle<T>(a, s, shat, kGateSecondHalf)) return false;
        with_width(lv.width, [&](auto W) {
            PSGB_SETS(lv, G) ph::bicg_t<T, decltype(W)::value, kPR>(lv, t0, G.gid, G.lane, shat, t, s, ctx);
        });
        PSGB_BARRIER(a);
        PSGB_SETS(lv, G) ph::bicg_x<T, kPR>(lv, t0, G.gid, G.lane, phat, shat, s, t, x, r, shadow, ctx);
        PSGB_BARRIER(a);
    }
    return true;
}

template <typename T>
__device__ bool pcg(const Args<T>& a) {
    const Group G = group_of();
    const LevelView<T>& lv = a.level[0].view;
    const ReduceCtx& ctx = a.ctx;
    T *r = a.k[0], *p = a.k[2], *q = a.k[3], *z = a.k[4];
    const T* rhs = a.k[8];
    T* x = a.k[9];
    const T omega_j = a.omega;
    T* z_first = pair_of(a, 0, z).first;
    PSGB_SETS(lv, G) ph::pcg_init<T, kPR>(lv, t0, G.gid, G.lane, rhs, x, r, p, z_first, omega_j, ctx, a.inner_tolerance, a.max_iterations);
    PSGB_BARRIER(a);
    if (!vcycle<T>(a, r, z, kGateRunning)) return false;
    for (int it = 0; it < a.max_iterations; ++it) {
        if (!any_inner_running(a.sc, a.instances)) break;
        PSGB_SETS(lv, G) ph::pcg_rz<T, kPR>(lv, t0, G.gid, G.lane, r, z, ctx);
        PSGB_BARRIER(a);
        PSGB_SETS(lv, G) ph::pcg_p<T, kPR>(lv, t0, G.lane, z, p, a.sc);
        PSGB_BARRIER(a);
        with_width(lv.width, [&](auto W) {
            PSGB_SETS(lv, G) ph::pcg_q<T, decltype(W)::value, kPR>(lv, t0, G.gid, G.lane, p, q, ctx);
        });
        PSGB_BARRIER(a);
        PSGB_SETS(lv, G) ph::pcg_xr<T, kPR>(lv, t0, G.gid, G.lane, p, q, x, r, z_first, omega_j, ctx);
        PSGB_BARRIER(a);
        if (!vcycle<T>(a, r, z, kGateRunning)) return false;
    }
    return true;
}

template <typename T>
__device__ bool refine(const Args<T>& a) {
    const Group G = group_of();
    const LevelView<double>& f = a.fine64;
    PSGB_SETS(f, G) ph::outer_init<kPR>(f, t0, G.gid, G.lane, a.rhs64, a.ctx, a.tolerance, a.active);
    PSGB_BARRIER(a);
    for (int round = 0; round <= a.max_refinements; ++round) {
        with_width(f.width, [&](auto W) {
            PSGB_SETS(f, G) ph::outer_residual<T, decltype(W)::value, kPR>(f, t0, G.gid, G.lane, a.rhs64, a.x64, a.r64, a.k[8], a.ctx, a.max_refinements);
        });
        PSGB_BARRIER(a);
        if (!any_outer_running(a.sc, a.instances)) break;
        if (!(a.method == kBiCGSTAB ? bicgstab<T>(a) : pcg<T>(a))) return false;
        if (blockIdx.x == 0) {
            for (unsigned i = threadIdx.x; i < a.instances; i += blockDim.x) ph::outer_account(a.sc[i]);
        }
        PSGB_BARRIER(a);
        PSGB_SETS(f, G) ph::outer_update<T, kPR>(f, t0, G.lane, a.k[9], a.x64, a.sc);
        PSGB_BARRIER(a);
    }
    return true;
}

template <typename T>
__global__ void __launch_bounds__(1024, 1) k_persistent_solve(const __grid_constant__ PersistentArgs<T> a) {
    refine<T>(a);
}

int blocks_per_sm(const void* kernel) {
    int per_sm = 0;
    PSGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 1024, 0));
    return per_sm;
}

}  // namespace

template <typename T>
int persistent_kernel_blocks_per_sm() {
    return blocks_per_sm(reinterpret_cast<const void*>(k_persistent_solve<T>));
}

template <typename T>
void persistent_kernel_launch(const PersistentArgs<T>& args, unsigned blocks, cudaStream_t st) {
    PersistentArgs<T> a = args;
    void* params[] = {&a};
    PSGB_LAUNCH(kFamPersistent, st,
                PSGB_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_persistent_solve<T>),
                                                      dim3(blocks), dim3(1024), params, 0, st)));
}

}  // namespace psgb
