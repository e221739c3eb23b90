// The coarse tail of the V-cycle (see coarse_tail.hpp): blocks of four 256-thread tile
// groups. A planet's groups walk its tiles of each level (group g of G takes tiles g,
// g + G, ...), call the shared per-tile phases, and meet at a barrier between phases (a
// block barrier, or with several blocks per planet a per-planet barrier in global
// memory); the dense coarsest solve gives one row to each of the planet's warps.
#define PSGB_PHASE_RESTRICT
#include "coarse_tail.hpp"
#include "phases.cuh"
#include "planet.hpp"
#include "profile.hpp"

#include <algorithm>
#include <stdexcept>
#include <string>
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

// The planet's tiles of level l, split over its `groups` tile groups (this one: `group`).
#define PSGB_PLANET_TILES(a, l, inst, group)                                                        \
    for (int tile = static_cast<int>((a).tile_range[((l) * (a).instances + (inst)) * 2]) + (group),   \
             tile_end = static_cast<int>((a).tile_range[((l) * (a).instances + (inst)) * 2] +        \
                                         (a).tile_range[((l) * (a).instances + (inst)) * 2 + 1]);     \
         tile < tile_end; tile += groups)

constexpr unsigned long long kTailBarrierTimeoutNs = 2000000000ull;   // 2 s
constexpr unsigned kTailSpinLimit = 1u << 26;

__device__ __forceinline__ unsigned ld_volatile_u(const unsigned* p) { return *reinterpret_cast<const volatile unsigned*>(p); }
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The `size` blocks of planet `inst` meet (sense by generation: the last to arrive resets
// the count and advances the generation). Every wait is bounded; past its limit the
// error flag is set and every block of the launch stops at its next barrier.
__device__ bool planet_barrier(unsigned* barrier, unsigned* error, unsigned instances, int inst, int size) {
    __shared__ int stop;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned* count = barrier + inst;
        unsigned* gen = barrier + instances + inst;
        const unsigned g = ld_volatile_u(gen);
        __threadfence();
        const unsigned arrived = atomicAdd(count, 1u);
        if (arrived == static_cast<unsigned>(size) - 1u) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const unsigned long long start = global_ns();
            unsigned spins = 0;
            while (ld_volatile_u(gen) == g) {
                if (ld_volatile_u(error) != 0u) break;
                ++spins;
                if (spins > kTailSpinLimit || ((spins & 1023u) == 0u && global_ns() - start > kTailBarrierTimeoutNs)) {
                    atomicExch(error, 1u);
                    break;
                }
                if (spins > 256u) __nanosleep(32);
            }
        }
        __threadfence();
        stop = ld_volatile_u(error) != 0u;
    }
    __syncthreads();
    return stop == 0;
}

// The tail's phases for planet `inst` (block `rank` of its `size` blocks).
template <typename T, bool Multi>
__device__ __forceinline__ void tail_body(const TailArgs<T>& a, int inst, int rank, int size) {
    const int gid = static_cast<int>(threadIdx.x >> 8), lane = static_cast<int>(threadIdx.x & 255);
    const int group = rank * ph::kGroups + gid, groups = size * ph::kGroups;
    const int coarsest = a.dense.level[inst];
    if (coarsest < a.first || !ph::gate_open(a.sc, inst, a.gate)) return;
    // between phases: the block, or all of the planet's blocks
#define PSGB_TAIL_SYNC()                                                                   \
    do {                                                                                   \
        if (Multi) {                                                                       \
            if (!planet_barrier(a.barrier, a.error, a.instances, inst, size)) return;      \
        } else {                                                                           \
            __syncthreads();                                                               \
        }                                                                                  \
    } while (0)
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
                    PSGB_PLANET_TILES(a, l, inst, group)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, gid, lane, L.b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, a.gate);
                } else {
                    PSGB_PLANET_TILES(a, l, inst, group)
                        ph::smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, p.second, omega, a.sc, a.gate);
                }
            });
            PSGB_TAIL_SYNC();
            T* t = p.first; p.first = p.second; p.second = t;
        }
        tail_widths(lv.width, [&](auto W) {
            PSGB_PLANET_TILES(a, l, inst, group)
                ph::residual<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, L.r, a.sc, a.gate);
        });
        PSGB_TAIL_SYNC();
        const PersistentLevel<T>& C = a.level[l + 1];
        const TailPair<T> pc = tail_pair(a, l + 1);
        PSGB_PLANET_TILES(a, l + 1, inst, group)
            ph::restrict_zero<T, 1>(C.view, tile, lane, L.member_offset, L.member, L.r, C.b, pc.first, omega, a.sc, a.gate);
        PSGB_TAIL_SYNC();
    }
    // The planet's coarsest level: x = A^-1 b, one warp per row.
    {
        const int n = static_cast<int>(a.dense.size[inst]);
        const PersistentLevel<T>& L = a.level[coarsest];
        for (int row = rank * 32 + static_cast<int>(threadIdx.x >> 5); row < n; row += 32 * size)
            ph::dense_row<T>(a.dense, inst, row, static_cast<int>(threadIdx.x & 31), a.dense_inv, L.b, L.x);
        PSGB_TAIL_SYNC();
    }
    // Up: prolongation fused with the first post-sweep, then the remaining post-sweeps.
    for (int l = coarsest - 1; l >= a.first; --l) {
        const PersistentLevel<T>& L = a.level[l];
        const LevelView<T>& lv = L.view;
        const T* e = a.level[l + 1].x;
        TailPair<T> p = tail_pair(a, l);
        if ((a.pre[l] - 1) & 1) { T* t = p.first; p.first = p.second; p.second = t; }   // where the down sweeps ended
        if (a.post[l] == 0) {
            PSGB_PLANET_TILES(a, l, inst, group) ph::prolong<T, 1>(lv, tile, lane, L.agg, e, p.first, a.sc, a.gate);
            PSGB_TAIL_SYNC();
            continue;
        }
        tail_widths(lv.width, [&](auto W) {
            PSGB_PLANET_TILES(a, l, inst, group)
                ph::prolong_smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.agg, e, L.b, p.first, p.second, omega, a.sc,
                                                             a.gate);
        });
        PSGB_TAIL_SYNC();
        { T* t = p.first; p.first = p.second; p.second = t; }
        for (int k = 1; k < a.post[l]; ++k) {
            tail_widths(lv.width, [&](auto W) {
                if (a.inner[l] > 1) {
                    PSGB_PLANET_TILES(a, l, inst, group)
                        ph::smooth_block<T, decltype(W)::value>(lv, tile, gid, lane, L.b, p.first, p.second, omega,
                                                                a.inner[l], a.sc, a.gate);
                } else {
                    PSGB_PLANET_TILES(a, l, inst, group)
                        ph::smooth<T, decltype(W)::value, 1>(lv, tile, lane, L.b, p.first, p.second, omega, a.sc, a.gate);
                }
            });
            PSGB_TAIL_SYNC();
            T* t = p.first; p.first = p.second; p.second = t;
        }
    }
#undef PSGB_TAIL_SYNC
}

template <typename T, bool Multi>
__global__ void __launch_bounds__(1024, 1) k_coarse_tail(const __grid_constant__ TailArgs<T> a) {
    pdl_begin();
    int inst = static_cast<int>(blockIdx.x), rank = 0, size = 1;
    if (Multi) {
        const std::uint32_t w = a.cta[blockIdx.x];
        inst = static_cast<int>(w & 0xFFFFu);
        rank = static_cast<int>((w >> 16) & 0xFFu);
        size = static_cast<int>(w >> 24);
    }
    tail_body<T, Multi>(a, inst, rank, size);
}

// One block per planet with the tail levels' vectors (x, y, b, r of every level from the
// tail level down) in shared memory: every phase's gathers, restrictions and prolongations
// then read shared memory, and only the matrix streams from L2. The level pointers of a
// copy of the arguments are rebased onto the planet's slices (vector[row] of a global row
// lands in the slice), so the phases run unchanged and give the same bits. In: the tail
// level's right-hand side and the iterate of its zero-start sweep; out: its final iterate.
template <typename T>
__global__ void __launch_bounds__(1024, 1) k_coarse_tail_shared(const __grid_constant__ TailArgs<T> a) {
    pdl_begin();
    const int inst = static_cast<int>(blockIdx.x);
    const int coarsest = a.dense.level[inst];
    if (coarsest < a.first || !ph::gate_open(a.sc, inst, a.gate)) return;
    extern __shared__ __align__(16) unsigned char tail_shared_bytes[];
    __shared__ TailArgs<T> la;
    __shared__ unsigned total;
    T* vec = reinterpret_cast<T*>(tail_shared_bytes);
    if (threadIdx.x == 0) {
        la = a;
        std::size_t off = 0;
        for (int l = a.first; l <= coarsest; ++l) {
            const std::size_t base = std::size_t(a.tile_range[(l * a.instances + inst) * 2]) * kTile;
            const std::size_t rows = std::size_t(a.tile_range[(l * a.instances + inst) * 2 + 1]) * kTile;
            T* slice = vec + off;
            la.level[l].x = slice - base;
            la.level[l].y = slice + rows - base;
            la.level[l].b = slice + 2 * rows - base;
            la.level[l].r = slice + 3 * rows - base;
            off += 4 * rows;
        }
        total = static_cast<unsigned>(off);
    }
    __syncthreads();
    for (unsigned i = threadIdx.x; i < total; i += blockDim.x) vec[i] = T(0);
    __syncthreads();
    const int first = a.first;
    const int t0 = static_cast<int>(a.tile_range[(first * a.instances + inst) * 2]);
    const int nt = static_cast<int>(a.tile_range[(first * a.instances + inst) * 2 + 1]);
    {
        const T* gx = tail_pair(a, first).first;
        T* sx = tail_pair(la, first).first;
        for (int row = t0 * kTile + static_cast<int>(threadIdx.x); row < (t0 + nt) * kTile; row += blockDim.x) {
            la.level[first].b[row] = a.level[first].b[row];
            sx[row] = gx[row];
        }
    }
    __syncthreads();
    tail_body<T, false>(la, inst, 0, 1);
    __syncthreads();
    for (int t = t0; t < t0 + nt; ++t) {
        const int rows = static_cast<int>((a.level[first].view.tile_meta[t] >> 22) & 0x1FFu);
        const int row = t * kTile + static_cast<int>(threadIdx.x);
        if (static_cast<int>(threadIdx.x) < rows) a.level[first].x[row] = la.level[first].x[row];
    }
}

}  // namespace


unsigned tail_block_budget() {
    int device = 0, coop = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || coop == 0) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_coarse_tail<float, true>, 1024, 0) != cudaSuccess)
        return 0;
    int per_sm64 = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm64, k_coarse_tail<double, true>, 1024, 0) != cudaSuccess)
        return 0;
    return static_cast<unsigned>(sms * std::min(per_sm, per_sm64));
}

template <typename T>
unsigned tail_shared_max_bytes() {
    // the block's opt-in shared memory less the kernel's static shared memory (its copy of
    // the arguments, the block-local sweeps' tiles); the kernel is opted in to it once
    static const unsigned limit = [] {
        int device = 0, optin = 0;
        cudaFuncAttributes fa{};
        if (cudaGetDevice(&device) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
            cudaFuncGetAttributes(&fa, k_coarse_tail_shared<T>) != cudaSuccess) {
            cudaGetLastError();
            return 0u;
        }
        const long room = static_cast<long>(optin) - static_cast<long>(fa.sharedSizeBytes);
        if (room <= 0) return 0u;
        if (cudaFuncSetAttribute(k_coarse_tail_shared<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(room)) != cudaSuccess) {
            cudaGetLastError();
            return 0u;
        }
        return static_cast<unsigned>(room);
    }();
    return limit;
}
template unsigned tail_shared_max_bytes<float>();
template unsigned tail_shared_max_bytes<double>();

template <typename T>
void launch_coarse_tail(const TailArgs<T>& args, cudaStream_t st) {
    if (args.cluster != 0) {
        launch_coarse_cluster<T>(args, st);
        return;
    }
    if (args.shared_rows != 0) {
        const std::size_t bytes = std::size_t(4) * args.shared_rows * sizeof(T);
        if (bytes > tail_shared_max_bytes<T>()) throw std::logic_error("coarse tail: the levels do not fit in shared memory");
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(args.instances);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = bytes;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = args.instances <= kPdlMaxBlocks ? 1 : 0;
        PSGB_LAUNCH(kFamSmoothCoarse, st, {
            const cudaError_t e = cudaLaunchKernelEx(&cfg, k_coarse_tail_shared<T>, args);
            if (e != cudaSuccess) throw std::runtime_error(std::string("coarse tail launch: ") + cudaGetErrorString(e));
        });
        return;
    }
    if (args.cta == nullptr) {
        PSGB_LAUNCH(kFamSmoothCoarse, st, launch_pdl(k_coarse_tail<T, false>, args.instances, 1024, st, args));
        return;
    }
    // Cooperative: every block co-resident (checked by the runtime), no early start.
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(args.ctas);
    cfg.blockDim = dim3(1024);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PSGB_LAUNCH(kFamSmoothCoarse, st, {
        const cudaError_t e = cudaLaunchKernelEx(&cfg, k_coarse_tail<T, true>, args);
        if (e != cudaSuccess) throw std::runtime_error(std::string("coarse tail launch: ") + cudaGetErrorString(e));
    });
}

template void launch_coarse_tail<float>(const TailArgs<float>&, cudaStream_t);
template void launch_coarse_tail<double>(const TailArgs<double>&, cudaStream_t);

}  // namespace psgb
