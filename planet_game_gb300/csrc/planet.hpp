// Internal (non-ABI) structures of the GB300 heat-transport library.
//
// Planet  : one mesh (level, radius) with its transport graph and multigrid
//           hierarchy structure, the operator geometry resident in HBM.
// Batch   : any number of planets concatenated level by level, each planet's rows
//           padded to whole 256-row tiles, with the Krylov/V-cycle workspace. A
//           one-planet batch is the plain drop-in solve; a many-planet batch is
//           the concatenated block layout solved by one stream of launches.
#pragma once

#include "host/hierarchy.hpp"
#include "host/mesh.hpp"
#include "kernels.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <tuple>
#include <stdexcept>
#include <string>
#include <vector>

namespace psgb {

constexpr std::uint32_t kTileRows = 256;

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define PSGB_CUDA(call)                                                                    \
    do {                                                                                   \
        cudaError_t psgb_err_ = (call);                                                    \
        if (psgb_err_ != cudaSuccess) {                                                    \
            throw ::psgb::CudaError(std::string(#call) + ": " + cudaGetErrorString(psgb_err_)); \
        }                                                                                  \
    } while (0)

// Device allocations owned by one object; counts bytes for the HBM budget.
class DeviceStore {
  public:
    DeviceStore() = default;
    DeviceStore(const DeviceStore&) = delete;
    DeviceStore& operator=(const DeviceStore&) = delete;
    ~DeviceStore() { release(); }
    template <typename T>
    T* alloc(std::size_t count) {
        if (count == 0) count = 1;
        void* p = nullptr;
        const std::size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
        if (arena_ != nullptr) {
            // Sub-allocation from caller-provided device memory: no allocation call.
            if (bytes > arena_capacity_ - bytes_) {
                throw std::invalid_argument("the no-allocation scratch (" + std::to_string(arena_capacity_) +
                                            " bytes) is too small for this planet");
            }
            p = arena_ + bytes_;
            bytes_ += bytes;
            return static_cast<T*>(p);
        }
        PSGB_CUDA(cudaMalloc(&p, bytes));
        ptrs_.push_back(p);
        bytes_ += bytes;
        return static_cast<T*>(p);
    }
    // Serve every later alloc() from [base, base + capacity) (256-byte aligned) instead
    // of cudaMalloc; release() then frees nothing.
    void use_arena(void* base, std::size_t capacity) {
        arena_ = static_cast<char*>(base);
        arena_capacity_ = capacity;
        bytes_ = 0;
    }
    bool arena() const { return arena_ != nullptr; }
    template <typename T>
    T* upload(const std::vector<T>& host) {
        T* d = alloc<T>(host.size());
        if (!host.empty()) PSGB_CUDA(cudaMemcpy(d, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
        return d;
    }
    void release() {
        for (void* p : ptrs_) cudaFree(p);
        ptrs_.clear();
        bytes_ = 0;
    }
    std::size_t bytes() const { return bytes_; }

  private:
    std::vector<void*> ptrs_;
    std::size_t bytes_ = 0;
    char* arena_ = nullptr;
    std::size_t arena_capacity_ = 0;
};

// Fine-level operator geometry, ELL slot-major over P = pad_rows(N) rows.
struct DevMesh {
    std::uint32_t n = 0, p = 0, edges = 0;
    std::int32_t* nbr = nullptr;       // [6][P]; padding slot -> own row
    std::int32_t* edge = nullptr;      // [6][P]; padding slot -> 0 (masked)
    std::uint8_t* first = nullptr;     // [P] bit j: this cell is edge slot j's first cell
    std::uint8_t* degree = nullptr;    // [P]
    double* w = nullptr;               // [6][P] l/d; 0 in padding slots
    double* dist = nullptr;            // [6][P] centroid distance; 1 in padding slots
    float* ne = nullptr;               // [6][P] FP32 outward normal (east)
    float* nn = nullptr;               // [6][P] FP32 outward normal (north)
    double* area = nullptr;            // [P] mesh cell areas; 1 in padding rows
    double* graph_area = nullptr;      // [P] the transport graph's node areas (differ when agglomerated)
    double* gm = nullptr;              // [4][P] m_ee, m_en, m_nn, det of the LSQ gradient
    double* edge_length = nullptr;     // [E]
    double* latitude = nullptr;        // [2][P] sin and cos of the cell centre's latitude
    // agglomerated planets: fine cells -> nodes
    std::uint32_t fine_cells = 0;
    std::uint32_t* group_of_cell = nullptr;   // [fine cells]
    std::uint32_t* member_offset = nullptr;   // [n + 1]: each node's fine cells ...
    std::uint32_t* member = nullptr;          // ... in cell order
    double* fine_area = nullptr;              // [fine cells]
};

struct Planet {
    HostMesh mesh;                     // for an agglomerated planet: the mesh one level coarser
    TransportGraph graph;              // ... and its graph with the groups' summed fine areas
    std::vector<std::uint32_t> group_of_cell;   // agglomerated planets: fine cell -> node
    std::vector<std::uint32_t> member_offset, member;   // ... each node's fine cells in cell order
    std::vector<double> fine_area_m2;  // ... the fine cells' areas
    std::size_t fine_cells = 0;        // agglomerated planets: cells of the fine mesh
    HostHierarchy hierarchy;
    DevMesh dev;
    DeviceStore store;
    bool uploaded = false;
    std::unique_ptr<struct Batch> solo;   // the one-planet batch (drop-in calls)
};

// One level of the concatenated hierarchy.
struct BatchLevel {
    std::uint32_t rows = 0;            // padded total P
    std::uint32_t tiles = 0;
    std::uint32_t width = 0;           // device ELL width (6, 8, 12, 16)
    std::int32_t* col = nullptr;       // [width][P]
    // planet-local columns once per distinct graph of the level's planets (null when no two
    // planets share one): [width][spitch], and per tile (planet's first row, that row
    // minus its graph's first row in scol)
    std::int32_t* scol = nullptr;
    int2* tile_shift = nullptr;
    std::uint32_t spitch = 0;
    double* vd64 = nullptr;            // [width][P] off-diagonals, then [P] diagonal
    double* inv64 = nullptr;           // [P] 1 / diagonal
    float* vd32 = nullptr;
    float* inv32 = nullptr;
    std::int32_t* tile_inst = nullptr;    // [tiles]
    std::int32_t* tile_rows = nullptr;    // [tiles] valid rows (0..256)
    std::uint8_t* tile_sweep = nullptr;   // [tiles] 1: the planet smooths on this level
    std::uint32_t* tile_meta = nullptr;   // [tiles rounded up to 4] pack_tile(inst, rows, sweep)
    std::uint8_t sets_stencil = 1;        // tiles per tile set of the level's launches (tuned)
    std::uint8_t sets_vector = 1;
    // transition to the next level (absent on the deepest level)
    std::int32_t* agg = nullptr;              // [P] global row on the next level
    std::uint32_t* member_offset = nullptr;   // next level: [P_next + 1]
    std::uint32_t* member = nullptr;
    std::uint32_t* gal_offset = nullptr;      // next level: [(width_next + 1) * P_next + 1]
    std::uint32_t* gal_source = nullptr;
    std::uint32_t gal_lists = 0;
    // vectors (x: iterate, y: Jacobi ping-pong, b: right-hand side, r: residual)
    double* x64 = nullptr; double* y64 = nullptr; double* b64 = nullptr; double* r64 = nullptr;
    float* x32 = nullptr; float* y32 = nullptr; float* b32 = nullptr; float* r32 = nullptr;
    std::vector<std::int64_t> base;    // [instances] row base, -1 if the planet has no such level
    std::vector<std::uint32_t> count;  // [instances] rows
};

struct DenseCoarse {
    std::vector<std::int32_t> level;   // coarsest level per planet
    std::vector<std::uint64_t> offset; // inverse offset per planet
    std::vector<std::uint32_t> size;
    std::vector<std::int64_t> row_base;
    std::uint32_t max_rows = 0;
    // per level: blocks of eight coarsest rows, (planet, first row), for the dense solves
    std::vector<std::uint32_t> block_offset;   // [levels + 1] into d_blocks
    int2* d_blocks = nullptr;
    double* inv64 = nullptr;           // concatenated row-major inverses
    float* inv32 = nullptr;
    double* work = nullptr;
    std::int32_t* d_level = nullptr;
    std::uint64_t* d_offset = nullptr;
    std::uint32_t* d_size = nullptr;
    std::int64_t* d_row_base = nullptr;
};

struct GraphKey {
    int precision_bytes, method, iterations;
    std::vector<int> shape;            // per level: pre, post sweeps and tile-set sizes
    double omega;
    double correction;
    bool operator<(const GraphKey& o) const {
        return std::tie(precision_bytes, method, iterations, shape, omega, correction) <
               std::tie(o.precision_bytes, o.method, o.iterations, o.shape, o.omega, o.correction);
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::uint64_t kernels = 0;
};

struct SmootherConfig {
    int pre = 2, post = 2;             // damped Jacobi sweeps on every level ...
    double omega = 0.8;                // damping factor
    // Scale of the coarse-grid correction (x += correction * P e). Plain aggregation
    // under-corrects smooth error; a scale of 1.5 to 2 (over-correction) cuts the Krylov
    // iterations by a quarter to a third on these hierarchies. 1: the plain V-cycle.
    double correction = 1.0;
    std::vector<int> level_pre, level_post;   // ... unless set per level (a tuning)
    std::vector<int> level_inner;             // per level: block-local sweeps per smoothing launch (1: plain Jacobi)
    int pre_at(std::size_t l) const { return l < level_pre.size() ? level_pre[l] : pre; }
    int post_at(std::size_t l) const { return l < level_post.size() ? level_post[l] : post; }
    int inner_at(std::size_t l) const { return l < level_inner.size() ? level_inner[l] : 1; }
    // The first (zero-start) sweep of level l writes x when the level's sweep count after
    // it is even, so that its last sweep ends in x.
    bool starts_in_x(std::size_t l) const { return ((pre_at(l) - 1 + post_at(l)) % 2) == 0; }
};

struct Batch {
    std::vector<Planet*> planets;
    std::uint32_t instances = 0;
    std::vector<BatchLevel> levels;
    DenseCoarse dense;
    DeviceStore store;
    SmootherConfig smoother;
    // Levels from tail_level down run as one block per planet (coarse_tail.hpp); 0: none.
    int tail_level = 0;
    int default_tail_level = 0;
    // Several co-resident blocks per large planet in the tail (cooperative launch): per
    // tail level the packed per-block words and their count (null: one block per planet).
    bool tail_spread = true;
    // One block per planet with the tail levels' vectors in shared memory (wins over spread);
    // per tail level the largest planet's padded rows summed down to its coarsest level.
    bool tail_shared = false;
    // A thread-block cluster of this many blocks per planet (2, 4 or 8; 0: none) with the
    // tail levels' vectors in the cluster's distributed shared memory (wins over both).
    unsigned tail_cluster = 0;
    // Blocks of the tail launch last built (0: none built under the current settings).
    unsigned tail_launch_blocks = 0;
    std::vector<unsigned> tail_rows_at;
    std::vector<std::uint32_t*> tail_cta_at;
    std::vector<unsigned> tail_ctas_at;
    unsigned* tail_barrier = nullptr;  // [2][instances]
    std::uint32_t* tile_range = nullptr;   // [levels][instances][2]: first tile, tile count
    bool tuned = false;                // per-level settings from an autotune: the options' sweeps do not apply
    std::vector<std::int64_t> fine_base;      // fine-level row base per planet
    // fine-level graph data for assembly and the transport operator
    double* area = nullptr;            // [P0]; 1 in padding rows
    double* w = nullptr;               // [6][P0] graph weight l/d (0 in padding slots)
    double* wsum = nullptr;            // [P0] the graph's weight_sum
    double* conductance = nullptr;     // [instances] scratch for assembly
    // Krylov vectors on the fine level
    static constexpr int kVectors = 10;
    double* k64[kVectors] = {};
    float* k32[kVectors] = {};
    // FP64 refinement
    double* xr = nullptr;              // solution
    double* rr = nullptr;              // residual
    double* bb = nullptr;              // right-hand side
    double* tmp = nullptr;             // [P0] general scratch
    double* tmp2 = nullptr;            // [P0] general scratch
    // reductions
    double* partial = nullptr;         // [tiles0][8]
    unsigned* ticket = nullptr;        // [instances]
    std::uint32_t* tile_begin = nullptr;  // [instances + 1] fine-level tile ranges
    InstanceScalars* scalars = nullptr;   // [instances]
    unsigned* sync = nullptr;          // [4] grid-barrier state of the persistent solve; [3]: tail barrier error
    std::vector<InstanceScalars> host_scalars;
    InstanceScalars* pinned_scalars = nullptr;   // pinned host mirror
    bool matrix_ready = false;
    std::vector<char> dense_at;        // [levels] some planet's coarsest level is this one
    // private stream of the solver (captured into CUDA graphs), fenced with the caller's
    cudaStream_t stream = nullptr;
    cudaEvent_t fence_in = nullptr, fence_out = nullptr;
    std::map<GraphKey, GraphEntry> graphs;
    bool use_graphs = true;
    // transport-step buffers (fine layout)
    double* slope_of = nullptr;        // [instances] dt / C
    double* t0 = nullptr;              // [P0]
    double* src = nullptr;             // [P0]
    double* hout = nullptr;            // [P0]
    double* tnew = nullptr;            // [P0]
    double* sums = nullptr;            // [instances][8]
    std::uint8_t* active = nullptr;    // [instances] planets taking part in the current step
    std::vector<std::uint8_t> host_active;
    bool active_mask = false;          // some planet is left out of the current step
    double* edge_g = nullptr;          // [6][P0] per-entry conductance (lazily)
    double* slope_field = nullptr;     // [P0] dt / C per row of the assembled matrix (lazily)
    bool reassemble = false;           // assemble on every step, even with unchanged parameters
    const double* step_edge_conductance = nullptr;   // edge_g when the matrix uses it
    double* csr_values = nullptr;      // one-planet batches: set_matrix staging
    std::uint32_t* csr_offset = nullptr;   // one-planet batches: the graph's CSR offsets
    // the parameters the current matrix was assembled with
    std::vector<double> assembled_key;                  // C, dt, K and the conductance source per planet
    std::vector<std::vector<double>> assembled_edges;   // per planet: per-edge conductance passed in (empty: none)
    std::vector<std::vector<double>> stored_edges;      // per planet: set with psgb_batch_set_edge_conductance
    std::vector<std::uint64_t> stored_generation;       // per planet: bumped on every set
    std::uint64_t assembled_bytes_hint = 0;
    ~Batch() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second.exec);
        if (fence_in != nullptr) cudaEventDestroy(fence_in);
        if (fence_out != nullptr) cudaEventDestroy(fence_out);
        if (stream != nullptr) cudaStreamDestroy(stream);
        if (pinned_scalars != nullptr) cudaFreeHost(pinned_scalars);
    }
};

}  // namespace psgb
