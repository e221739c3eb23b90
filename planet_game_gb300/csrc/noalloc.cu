// A transport step that allocates nothing: psgb_transport_step_noalloc.
//
// Who needs it: callers that must not call cudaMalloc (or any other allocating CUDA
// routine) while they run - a simulation loop that reserved a fixed memory budget up
// front and may not grow it, a host that lends this library a GPU it shares under a hard
// memory cap, or a plugin host whose own allocator owns the device memory. The regular
// entry points allocate a planet's device workspace on first use; this one never does.
//
// How: every device array the solver needs (matrix hierarchy, Krylov and V-cycle
// vectors, reduction partials) is placed in one file-scope device array,
// g_noalloc_scratch, of kNoAllocScratchBytes (8 MiB). Every GPU that loads this library
// holds that array until the process exits. The host cannot use the array's name as an
// address (in host code it is only a stand-in), so the first call on each device, with
// that device current, looks the address up with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture. Planets of at most kNoAllocMaxCells cells
// (10,242: a level-5 mesh) fit; larger ones are rejected with PSGB_ERR_INVALID_ARGUMENT.
// A per-edge conductance passed with the call is laid into the same array; the stored
// conductance of a batch (psgb_batch_set_edge_conductance) does not exist here and is
// rejected. No graphs, streams, events or pinned buffers are created: the work runs on
// the caller's stream, and the call waits for that stream before it returns (the solver's
// scalars come back through pageable copies).
//
// CUDA loads kernels lazily by default: the first call on a device, and the first call
// of each precision, load their kernels and map the array. Make one warm-up call per
// precision (or run with CUDA_MODULE_LOADING=EAGER) before relying on the no-allocation
// property.
//
// The array is shared by every call on a device and keeps the last call's contents;
// the step clears what must start at zero (reduction tickets, solver state) itself.
// Calls that overlap on the GPU (two streams, two threads) race on the array: serialise
// them.
#include "capi_internal.hpp"

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>

namespace {

constexpr std::size_t kNoAllocScratchBytes = std::size_t(8) << 20;
constexpr std::uint64_t kNoAllocMaxCells = 10242;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct DeviceScratch {
    void* address = nullptr;                 // device address of g_noalloc_scratch
    std::uint64_t owner = 0;                 // serial of the planet laid out in it
    std::unique_ptr<psgb::Batch> batch;      // host bookkeeping of that layout
};

std::mutex g_mutex;
std::map<int, DeviceScratch> g_devices;      // by device ordinal

// Set-up, once per device, with that device current.
DeviceScratch& scratch_for_current_device() {
    int device = 0;
    PSGB_CUDA(cudaGetDevice(&device));
    DeviceScratch& d = g_devices[device];
    if (d.address == nullptr) {
        void* ptr = nullptr;
        PSGB_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        d.address = ptr;
    }
    return d;
}

}  // namespace

using namespace psgb::capi;

extern "C" int psgb_transport_step_noalloc(psgb_planet* planet, const psgb_step_params* params,
                                           const psgb_solve_options* options, const double* t0_K,
                                           const double* source_W_m2, double* t_new_K, double* transport_W_m2,
                                           psgb_step_report* report, void* stream) {
    return guarded([&] {
        if (planet == nullptr || params == nullptr || t0_K == nullptr || source_W_m2 == nullptr || t_new_K == nullptr) {
            throw std::invalid_argument("null argument");
        }
        if (params->edge_conductance_stored) {
            throw std::invalid_argument("psgb_transport_step_noalloc has no stored per-edge conductance: pass the "
                                        "array in edge_conductance");
        }
        const std::uint64_t cells = planet->planet->mesh.cells;
        if (cells > kNoAllocMaxCells) {
            throw std::invalid_argument("psgb_transport_step_noalloc handles planets of at most 10242 cells "
                                        "(a level-5 mesh); this one has " + std::to_string(cells));
        }
        const psgb::SolveOptions opt = to_options(options);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        std::lock_guard<std::mutex> lock(g_mutex);
        DeviceScratch& d = scratch_for_current_device();
        if (d.owner != planet->serial || !d.batch) {
            d.batch.reset();
            d.owner = 0;
            d.batch = psgb::make_batch_in({planet->planet.get()}, d.address, kNoAllocScratchBytes);
            d.owner = planet->serial;
        }
        psgb::Batch& b = *d.batch;
        apply_smoother(b, options);
        PSGB_CUDA(cudaMemsetAsync(b.ticket, 0, b.instances * sizeof(unsigned), st));
        assemble_step_matrix(b, params, st);
        const std::size_t n = cells;
        PSGB_CUDA(cudaMemcpyAsync(b.t0, t0_K, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        PSGB_CUDA(cudaMemcpyAsync(b.src, source_W_m2, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        run_step(b, opt, st);
        PSGB_CUDA(cudaMemcpyAsync(t_new_K, b.tnew, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        if (transport_W_m2 != nullptr) {
            PSGB_CUDA(cudaMemcpyAsync(transport_W_m2, b.hout, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
        psgb_step_report local;
        step_reports(b, &local, st);
        if (report != nullptr) *report = local;
        if (local.solve.status != PSGB_OK) g_last_error = status_message(local.solve.status);
        return local.solve.status;
    });
}
