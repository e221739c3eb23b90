// Internal declarations shared by the C-ABI translation units (capi.cpp, noalloc.cu).
#pragma once

#include "../../include/planetsim_gb300.h"
#include "multirhs.hpp"
#include "solver.hpp"

#include <cstdint>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace psgb {

struct NonsymContext;   // the non-symmetric solves' per-planet structures (nonsym.cu)

// A numerical breakdown reported as PSGB_ERR_BREAKDOWN (a zero ILU pivot).
struct Breakdown : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Page-locked host doubles (the Newton solve's copies of h, T and dT/dh).
class PinnedDoubles {
  public:
    PinnedDoubles() = default;
    PinnedDoubles(const PinnedDoubles&) = delete;
    PinnedDoubles& operator=(const PinnedDoubles&) = delete;
    ~PinnedDoubles() {
        if (p_ != nullptr) cudaFreeHost(p_);
    }
    void reset(std::size_t count) {
        if (p_ != nullptr) cudaFreeHost(p_);
        p_ = nullptr;
        PSGB_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p_), count * sizeof(double)));
    }
    double* data() const { return p_; }

  private:
    double* p_ = nullptr;
};

}  // namespace psgb

struct psgb_planet {
    std::unique_ptr<psgb::Planet> planet;
    // lazily created device staging for host-memory calls
    psgb::DeviceStore stage_store;
    std::vector<double*> stage;
    std::size_t stage_len = 0;
    std::uint64_t serial = 0;   // unique per planet for the life of the process
    // the implicit transport solve's device vectors and pinned host copies
    psgb::DeviceStore newton_store;
    std::vector<double*> newton;
    psgb::PinnedDoubles newton_pinned;
    std::shared_ptr<psgb::NonsymContext> nonsym;
    // the multi-right-hand-side block solve's workspace and host-input staging
    std::unique_ptr<psgb::mr::Space> multi;
    std::vector<double*> multi_stage;
};

struct psgb_batch {
    std::unique_ptr<psgb::Batch> batch;
};

namespace psgb::capi {

extern thread_local std::string g_last_error;
int fail(int code, const std::string& message);

// Runs `body`, mapping the reference's exception families onto status codes.
template <typename F>
int guarded(F&& body) {
    try {
        g_last_error.clear();
        return body();
    } catch (const std::invalid_argument& e) {
        return fail(PSGB_ERR_INVALID_ARGUMENT, e.what());
    } catch (const psgb::Breakdown& e) {
        return fail(PSGB_ERR_BREAKDOWN, e.what());
    } catch (const std::bad_alloc& e) {
        return fail(PSGB_ERR_OUT_OF_MEMORY, e.what());
    } catch (const psgb::CudaError& e) {
        const std::string m = e.what();
        return fail(m.find("out of memory") != std::string::npos ? PSGB_ERR_OUT_OF_MEMORY : PSGB_ERR_CUDA, m);
    } catch (const std::overflow_error& e) {
        return fail(PSGB_ERR_INVALID_ARGUMENT, e.what());
    } catch (const std::logic_error& e) {
        return fail(PSGB_ERR_LOGIC, e.what());
    } catch (const std::exception& e) {
        return fail(PSGB_ERR_CUDA, e.what());
    }
}

psgb::SolveOptions to_options(const psgb_solve_options* o);
void apply_smoother(psgb::Batch& b, const psgb_solve_options* o);
int status_of(const psgb::InstanceScalars& s);
const char* status_message(int code);
void fill_report(const psgb::InstanceScalars& s, psgb_solve_report* r);
// Assemble (A/s + K L) on every planet unless the parameters equal the current ones.
void assemble_step_matrix(psgb::Batch& b, const psgb_step_params* params, cudaStream_t st);
// One transport step on every planet of a batch; inputs already in b.t0 / b.src.
void run_step(psgb::Batch& b, const psgb::SolveOptions& opt, cudaStream_t st);
void step_reports(psgb::Batch& b, psgb_step_report* reports, cudaStream_t st);

}  // namespace psgb::capi
