// Persistent cooperative solver: one launch per solve for every planet of a batch.
// (Host side; the kernel is in persistent_kernel.cuh, one translation unit per
// precision.)
//
// The kernel runs, device-side, what the one-kernel-per-phase path drives from the host
// (solver.cpp: solve, krylov, vcycle): the FP64 iterative refinement (residual, inner
// solve, update) around the inner BiCGSTAB or PCG iteration, and inside it the V-cycle
// over every multigrid level. Each phase is the same per-tile code as the kernel path
// (phases.cuh), so the arithmetic, and every result, is identical; between phases all
// blocks meet at a grid barrier instead of a kernel boundary. Planets that converged are
// masked per tile, as before; a loop ends when no planet is running, which every block
// decides identically from the device-resident per-planet scalars right after a barrier.
//
// Launch: cooperative (all blocks co-resident, checked by the runtime), one 1024-thread
// block per SM = four 256-row tile groups. The barrier polls a generation counter with a
// time and an iteration limit: past either the kernel records an error and every block
// returns at its next barrier, so no wait is unbounded.
#include "persistent.hpp"
#include "solver.hpp"

#include <map>
#include <mutex>
#include <stdexcept>

namespace psgb {

bool persistent_supported() {
    int device = 0, coop = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || coop == 0) return false;
    return persistent_kernel_blocks_per_sm<float>() >= 1 && persistent_kernel_blocks_per_sm<double>() >= 1;
}

namespace {

// Persistent solves on one device run one after another, whichever stream launched them:
// each waits for the previous one's completion event. Two grids that each wait for all of
// their blocks must never hold parts of the device at the same time.
std::mutex g_serial_mutex;
std::map<int, cudaEvent_t> g_serial_last;

}  // namespace

template <typename T>
void launch_persistent(const PersistentArgs<T>& args, cudaStream_t st, bool serialize) {
    if (args.depth < 1 || args.depth > kMaxLevels) throw std::logic_error("persistent solve: unsupported hierarchy depth");
    int device = 0, sms = 0;
    PSGB_CUDA(cudaGetDevice(&device));
    PSGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    if (persistent_kernel_blocks_per_sm<T>() < 1)
        throw std::runtime_error("persistent solve: a 1024-thread block does not fit an SM");
    std::unique_lock<std::mutex> lock(g_serial_mutex, std::defer_lock);
    cudaEvent_t* last = nullptr;
    if (serialize) {
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        PSGB_CUDA(cudaStreamIsCapturing(st, &capture));
        if (capture == cudaStreamCaptureStatusNone) {
            lock.lock();
            last = &g_serial_last[device];
            if (*last == nullptr) {
                PSGB_CUDA(cudaEventCreateWithFlags(last, cudaEventDisableTiming));
            } else {
                PSGB_CUDA(cudaStreamWaitEvent(st, *last, 0));
            }
        }
    }
    persistent_kernel_launch<T>(args, static_cast<unsigned>(sms), st);
    if (last != nullptr) PSGB_CUDA(cudaEventRecord(*last, st));
}

template void launch_persistent<float>(const PersistentArgs<float>&, cudaStream_t, bool);
template void launch_persistent<double>(const PersistentArgs<double>&, cudaStream_t, bool);

}  // namespace psgb
