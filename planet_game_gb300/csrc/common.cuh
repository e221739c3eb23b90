// Shared device-side helpers for the GB300 heat-transport kernels.
//
// Layout conventions used by every kernel:
//  * rows of a level are padded to a multiple of kTile (256) so that a tile -
//    the reference's deterministic 256-cell block (planet_mesh.hpp:76) - never
//    straddles two planets of a batch;
//  * neighbour data is ELL, slot-major: entry (slot j, row r) sits at j * P + r for a
//    level with padded row count P, so a warp reads 32 consecutive rows of one slot
//    (fully coalesced); rows with fewer neighbours pad with (column = row, value = 0);
//  * every reduction is deterministic: a fixed warp-shuffle tree inside a tile,
//    per-tile partials in global memory, and the last tile of a planet to finish
//    (integer ticket) sums that planet's partials in tile order.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <stdexcept>
#include <string>
#include <utility>

namespace psgb {

constexpr int kTile = 256;

// Programmatic dependent launch. Solve kernels run back to back on one stream, each
// short; launched with launch_pdl, a kernel's blocks may be scheduled while its
// predecessor drains. Every such kernel starts with pdl_begin(): it waits until the
// predecessor grid has completed and its writes are visible (so nothing is read early),
// then allows the successor to be scheduled. Measured on GB300 in CUDA graphs, early
// scheduling saves ~0.2 us per launch for grids of up to a few hundred blocks and costs
// up to 4 us for grids of thousands (their waiting blocks hold the SMs' block slots), so
// only grids of at most kPdlMaxBlocks blocks take it; pdl_begin() is free for the others.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

constexpr unsigned kPdlMaxBlocks = 1024;

template <typename... P, typename... A>
inline void launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, cudaStream_t st, A&&... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = grid.x * grid.y * grid.z <= kPdlMaxBlocks ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
    if (e != cudaSuccess) throw std::runtime_error(std::string("kernel launch: ") + cudaGetErrorString(e));
}

// Warp-level sum in a fixed butterfly order (result valid in every lane).
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over a 256-thread block in fixed order; result in thread 0.
// `scratch` holds 8 values per accumulated quantity.
template <typename T, int N>
__device__ __forceinline__ void block_sum256(T (&v)[N], T (*scratch)[8]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < N; ++q) {
        T w = warp_sum(v[q]);
        if (lane == 0) scratch[q][warp] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            T s = scratch[q][0];
#pragma unroll
            for (int w = 1; w < 8; ++w) s += scratch[q][w];
            v[q] = s;
        }
    }
}

// Double precision add/multiply that the compiler may not fuse into an FMA, for
// sums whose rounding must match the reference's sequential CPU loops.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

}  // namespace psgb
