// The implicit transport solve with a general tile response (sim/planet/surface/
// heat_transport.cpp:595-772, ImplicitTransportSettings and ImplicitTransportResult in
// heat_transport.hpp:82-119), with the Newton iterate resident in device memory.
//
// Find sources h with F(h) = h - K lap(T(h)) (+ latent) = 0, where T(h) and its slope dT/dh
// come from the response. Every vector of the iteration lives on the GPU: the response
// (a device callback, or the host callback behind pinned copies), the two-point
// Laplacians, the residual and its merit sum A F^2, the line search trials and the linear
// Newton systems (A/s - K Q) dT = -A F (multigrid-preconditioned Krylov). The host reads
// two scalars per evaluation, the merit and max |F|, and takes the reference's
// decisions: a backtracking line search on the merit with the iterate kept at or above
// the floor, a bounded number of full steps across kinks when no descent is found above
// the rounding floor, and the conservative flux form of the last iterate's temperatures
// as the transport applied. Sums reduce over 256-cell blocks in a fixed tree, then over
// the blocks in a fixed order: the same bits on every run.
//
// The file also holds the quartic column response of the reference's transport test as
// a kernel (test_heat_transport.cpp:30-76 over column_step.cpp:254-276), compiled
// without FMA contraction so that it reproduces the reference's roots bit for bit.
#include "../../include/planetsim_gb300.h"
#include "capi_internal.hpp"
#include "operators.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <utility>
#include <vector>

namespace {

using psgb::capi::guarded;

constexpr int kThreads = 256;   // one reduction block = 256 cells, as the reference's blocks

void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

unsigned blocks_of(std::size_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

// Fixed-shape tree sum / max over the block's 256 values.
__device__ double block_sum(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = sh[t] + sh[t + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}
__device__ double block_max(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = fmax(sh[t], sh[t + s]);   // NaN ignored, as std::max(largest, x)
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// h = max(0, floor).
__global__ void k_start(std::uint32_t n, const double* __restrict__ floor, double* __restrict__ source) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) source[i] = 0.0 < floor[i] ? floor[i] : 0.0;
}

// F = h - K lap T (+ latent); per block: sum A F^2 and max |F|.
__global__ void __launch_bounds__(kThreads) k_residual(std::uint32_t n, const double* __restrict__ h,
                                                       const double* __restrict__ diffusion,
                                                       const double* __restrict__ latent,
                                                       const double* __restrict__ area,
                                                       double* __restrict__ residual, double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    double merit = 0.0, largest = 0.0;
    if (i < n) {
        double r = h[i] - diffusion[i];
        if (latent != nullptr) r = r + latent[i];
        residual[i] = r;
        merit = area[i] * r * r;
        largest = fabs(r);
    }
    const double s = block_sum(merit, sh);
    const double m = block_max(largest, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * 3 + 0] = s;
        partial[blockIdx.x * 3 + 1] = m;
    }
}

// The final sums of the applied transport H: sum A H, sum |A H|, sum A H T.
__global__ void __launch_bounds__(kThreads) k_applied(std::uint32_t n, double* __restrict__ applied,
                                                      const double* __restrict__ latent,
                                                      const double* __restrict__ area,
                                                      const double* __restrict__ mean, double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    double flux = 0.0, dissipation = 0.0;
    if (i < n) {
        double H = applied[i];
        if (latent != nullptr) {
            H = H - latent[i];
            applied[i] = H;
        }
        flux = area[i] * H;
        dissipation = flux * mean[i];
    }
    const double a = block_sum(flux, sh);
    const double b = block_sum(fabs(flux), sh);
    const double c = block_sum(dissipation, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * 3 + 0] = a;
        partial[blockIdx.x * 3 + 1] = b;
        partial[blockIdx.x * 3 + 2] = c;
    }
}

// One block: the blocks' partials in a fixed order (thread t takes blocks t, t + 256, ...
// in order, then the tree); `max_mask` bit q: quantity q is a max.
__global__ void __launch_bounds__(kThreads) k_reduce(unsigned blocks, int quantities, unsigned max_mask,
                                                     const double* __restrict__ partial, double* __restrict__ out) {
    __shared__ double sh[kThreads];
    for (int q = 0; q < quantities; ++q) {
        const bool is_max = (max_mask >> q) & 1u;
        double v = 0.0;
        for (unsigned b = threadIdx.x; b < blocks; b += kThreads) {
            const double x = partial[b * 3 + q];
            v = is_max ? fmax(v, x) : v + x;
        }
        const double r = is_max ? block_max(v, sh) : block_sum(v, sh);
        if (threadIdx.x == 0) out[q] = r;
    }
}

// The Newton system's right-hand side -A F and a zero start.
__global__ void k_newton_rhs(std::uint32_t n, const double* __restrict__ residual, const double* __restrict__ area,
                             double* __restrict__ rhs, double* __restrict__ x) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) {
        rhs[i] = -residual[i] * area[i];
        x[i] = 0.0;
    }
}

// dh = K lap dT - F.
__global__ void k_direction(std::uint32_t n, const double* __restrict__ residual, double* __restrict__ delta) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) delta[i] = delta[i] - residual[i];
}

// trial = max(h + step dh, floor), keeping a NaN sum as std::max(sum, floor) does.
__global__ void k_trial(std::uint32_t n, const double* __restrict__ source, const double* __restrict__ delta,
                        double step, const double* __restrict__ floor, double* __restrict__ trial) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) {
        const double v = source[i] + step * delta[i];
        trial[i] = v < floor[i] ? floor[i] : v;
    }
}

// The root of a x + r x^4 = b (b > 0) by solve_column_surface's dry Newton
// (column_step.cpp:254-270): start at min(b/a, (b/r)^(1/4)), at most 10 steps, stop once
// a step is within 4 eps x.
__device__ double quartic_root(double a, double r, double b) {
    const double by_a = b / a, by_r = sqrt(sqrt(b / r));
    double x = by_r < by_a ? by_r : by_a;
    for (int iteration = 0; iteration < 10; ++iteration) {
        const double x3 = x * x * x;
        const double value = a * x + r * x3 * x - b;
        const double slope = a + 4.0 * r * x3;
        const double step = value / slope;
        x -= step;
        if (fabs(step) <= 4.0 * DBL_EPSILON * x) break;
    }
    return x;
}

// The test's response per cell c (test_heat_transport.cpp:41-56); `group` maps the cell
// to the node whose source it sees (null: itself).
__global__ void k_quartic(std::uint32_t n, double a, double r, const double* __restrict__ b,
                          std::uint32_t hold_stride, double hold_K, const std::uint32_t* __restrict__ group,
                          const double* __restrict__ source, double* __restrict__ mean, double* __restrict__ slope) {
    const std::uint32_t c = blockIdx.x * kThreads + threadIdx.x;
    if (c >= n) return;
    const double h = source[group != nullptr ? group[c] : c];
    const double x = quartic_root(a, r, b[c] + h);
    if (hold_stride != 0 && c % hold_stride == 0 && x > hold_K) {
        mean[c] = hold_K;
        slope[c] = 0.0;
        return;
    }
    mean[c] = x;
    slope[c] = 1.0 / (a + 4.0 * r * x * x * x);
}

#define PSGB_CHECK_LAUNCH() PSGB_CUDA(cudaGetLastError())

// The solve's device vectors, kept with the planet between calls.
struct Workspace {
    double *source, *mean, *slope, *residual, *trial, *trial_mean, *trial_slope, *trial_residual;
    double *delta_mean, *delta_source, *diffusion, *rhs, *floor, *latent, *partial, *scalars;
    double *host_source, *host_mean, *host_slope, *host_scalars;   // pinned
};

Workspace workspace(psgb_planet* h, std::size_t n) {
    if (h->newton.empty()) {
        const std::size_t blocks = blocks_of(n);
        for (int v = 0; v < 14; ++v) h->newton.push_back(h->newton_store.alloc<double>(n));
        h->newton.push_back(h->newton_store.alloc<double>(3 * blocks));
        h->newton.push_back(h->newton_store.alloc<double>(4));
        h->newton_pinned.reset(3 * n + 4);
    }
    double** v = h->newton.data();
    double* p = h->newton_pinned.data();
    return Workspace{v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12], v[13],
                     v[14], v[15], p, p + n, p + 2 * n, p + 3 * n};
}

struct Response {
    // device arrays on the solve's stream
    virtual void operator()(const double* h, double* mean, double* slope) = 0;
    virtual ~Response() = default;
};

struct Solver {
    psgb_planet* planet;
    std::size_t n;
    double K;
    const double* area;     // device: the graph's node areas
    const double* latent;   // device or null
    Response& response;
    psgb_solve_options inner;
    Workspace w;
    cudaStream_t st;

    void laplacian(const double* t, double* out) {
        const int code = psgb_diffusion_source(planet, K, t, out, PSGB_MEMORY_DEVICE, st);
        if (code != PSGB_OK) throw std::runtime_error(psgb_last_error());
    }

    // The response at h, F(h); returns the merit sum A F^2 and sets max |F|.
    double evaluate(const double* h, double* mean, double* slope, double* residual, double& largest) {
        response(h, mean, slope);
        laplacian(mean, w.diffusion);
        const unsigned blocks = blocks_of(n);
        k_residual<<<blocks, kThreads, 0, st>>>(static_cast<std::uint32_t>(n), h, w.diffusion, latent, area, residual,
                                               w.partial);
        PSGB_CHECK_LAUNCH();
        k_reduce<<<1, kThreads, 0, st>>>(blocks, 2, 0x2u, w.partial, w.scalars);
        PSGB_CHECK_LAUNCH();
        PSGB_CUDA(cudaMemcpyAsync(w.host_scalars, w.scalars, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        largest = w.host_scalars[1];
        return w.host_scalars[0];
    }

    // (A/s + K L) dT = -A F with held cells (s = 0) pinned at zero; Krylov iterations.
    int newton_system(const double* slope, const double* residual, double* dt) {
        k_newton_rhs<<<blocks_of(n), kThreads, 0, st>>>(static_cast<std::uint32_t>(n), residual, area, w.rhs, dt);
        PSGB_CHECK_LAUNCH();
        psgb_solve_report rep{};
        const int code = psgb_solve_newton_system(planet, &inner, K, slope, w.rhs, dt, &rep, PSGB_MEMORY_DEVICE, st);
        // An inexact inner solve is fine (the outer loop converges regardless); only a
        // failure that leaves no usable direction ends the solve.
        if (code != PSGB_OK && code != PSGB_ERR_NOT_CONVERGED) throw std::runtime_error(psgb_last_error());
        return rep.iterations;
    }

    void trial(const double* source, double step, double* out) {
        k_trial<<<blocks_of(n), kThreads, 0, st>>>(static_cast<std::uint32_t>(n), source, w.delta_source, step, w.floor,
                                                  out);
        PSGB_CHECK_LAUNCH();
    }
};

psgb_transport_settings checked_settings(const psgb_transport_settings* in) {
    psgb_transport_settings s;
    psgb_transport_settings_default(&s);
    if (in != nullptr) s = *in;
    require(s.max_newton_iterations >= 0 && s.max_line_search_halvings >= 0 && s.max_non_monotone_steps >= 0 &&
                s.max_cg_iterations > 0,
            "iteration limits must not be negative");
    require(s.cg_relative_tolerance > 0.0 && s.cg_relative_tolerance < 1.0, "the inner tolerance must be in (0, 1)");
    return s;
}

// The Newton iteration of heat_transport.cpp:620-772 on device vectors; the floor and
// latent heat are already in w.floor / w.latent.
psgb_transport_result newton(Solver& s, const psgb_transport_settings& settings) {
    Workspace& w = s.w;
    const std::uint32_t n = static_cast<std::uint32_t>(s.n);
    const unsigned blocks = blocks_of(s.n);
    double* source = w.source;
    double* mean = w.mean;
    double* slope = w.slope;
    double* residual = w.residual;
    double* trial = w.trial;
    double* trial_mean = w.trial_mean;
    double* trial_slope = w.trial_slope;
    double* trial_residual = w.trial_residual;
    k_start<<<blocks, kThreads, 0, s.st>>>(n, w.floor, source);
    PSGB_CHECK_LAUNCH();
    psgb_transport_result out{};
    double largest = 0.0;
    double merit = s.evaluate(source, mean, slope, residual, largest);
    int non_monotone = 0;
    for (int iteration = 0; iteration < settings.max_newton_iterations; ++iteration) {
        if (largest <= settings.newton_tolerance_W_m2) break;
        // Newton direction: dT from the linear system, dh = -F + K lap(dT).
        out.cg_iterations += s.newton_system(slope, residual, w.delta_mean);
        s.laplacian(w.delta_mean, w.delta_source);
        k_direction<<<blocks, kThreads, 0, s.st>>>(n, residual, w.delta_source);
        PSGB_CHECK_LAUNCH();
        // Backtracking on the merit; the iterate never drops below the floor.
        double step = 1.0, trial_merit = 0.0, trial_largest = 0.0;
        for (int halving = 0;; ++halving) {
            s.trial(source, step, trial);
            trial_merit = s.evaluate(trial, trial_mean, trial_slope, trial_residual, trial_largest);
            if (trial_merit < merit) break;
            if (halving == settings.max_line_search_halvings) {
                // No descent: at the rounding floor stop; farther out (a kink of the
                // response) take the full step a bounded number of times, unless it is
                // not finite or raises the merit too much.
                if (largest <= settings.rounding_floor_W_m2 || non_monotone == settings.max_non_monotone_steps) {
                    step = 0.0;
                } else {
                    ++non_monotone;
                    step = 1.0;
                    s.trial(source, 1.0, trial);
                    trial_merit = s.evaluate(trial, trial_mean, trial_slope, trial_residual, trial_largest);
                    if (!(std::isfinite(trial_merit) && trial_merit <= settings.max_non_monotone_growth * merit))
                        step = 0.0;
                }
                break;
            }
            step *= 0.5;
        }
        if (step == 0.0) break;
        std::swap(source, trial);
        std::swap(mean, trial_mean);
        std::swap(slope, trial_slope);
        std::swap(residual, trial_residual);
        merit = trial_merit;
        largest = trial_largest;
        ++out.newton_iterations;
    }
    // The transport applied: the conservative flux form of the last temperatures.
    s.laplacian(mean, w.diffusion);
    k_applied<<<blocks, kThreads, 0, s.st>>>(n, w.diffusion, s.latent, s.area, mean, w.partial);
    PSGB_CHECK_LAUNCH();
    k_reduce<<<1, kThreads, 0, s.st>>>(blocks, 3, 0x0u, w.partial, w.scalars);
    PSGB_CHECK_LAUNCH();
    PSGB_CUDA(cudaMemcpyAsync(w.host_scalars, w.scalars, 3 * sizeof(double), cudaMemcpyDeviceToHost, s.st));
    PSGB_CUDA(cudaStreamSynchronize(s.st));
    out.consistency_residual_W_m2 = largest;
    out.sum_W = w.host_scalars[0];
    out.absolute_sum_W = w.host_scalars[1];
    out.dissipation_W_K = w.host_scalars[2];
    // the results: H in w.diffusion, T in `mean` (copied out by the caller)
    w.source = w.diffusion;
    w.mean = mean;
    return out;
}

// The caller's host response behind pinned copies.
struct HostResponse final : Response {
    psgb_transport_response fn;
    void* user;
    std::size_t n;
    Workspace* w;
    cudaStream_t st;
    void operator()(const double* h, double* mean, double* slope) override {
        PSGB_CUDA(cudaMemcpyAsync(w->host_source, h, n * 8, cudaMemcpyDeviceToHost, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        if (fn(user, n, w->host_source, w->host_mean, w->host_slope) != 0)
            throw std::runtime_error("the transport response callback failed");
        PSGB_CUDA(cudaMemcpyAsync(mean, w->host_mean, n * 8, cudaMemcpyHostToDevice, st));
        PSGB_CUDA(cudaMemcpyAsync(slope, w->host_slope, n * 8, cudaMemcpyHostToDevice, st));
    }
};

struct DeviceResponse final : Response {
    psgb_device_response fn;
    void* user;
    std::size_t n;
    cudaStream_t st;
    void operator()(const double* h, double* mean, double* slope) override {
        if (fn(user, n, h, mean, slope, st) != 0) throw std::runtime_error("the transport response callback failed");
    }
};

struct Setup {
    std::size_t n;
    const double* area;
};

Setup setup(psgb_planet* planet) {
    psgb::upload_planet(*planet->planet);
    return Setup{planet->planet->mesh.cells, planet->planet->dev.graph_area};
}

void copy_vector(double* dst, const double* src, std::size_t n, int memory, bool in, cudaStream_t st) {
    const cudaMemcpyKind kind = memory == PSGB_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice
                                : in                         ? cudaMemcpyHostToDevice
                                                             : cudaMemcpyDeviceToHost;
    PSGB_CUDA(cudaMemcpyAsync(dst, src, n * 8, kind, st));
}

}  // namespace

extern "C" {

void psgb_transport_settings_default(psgb_transport_settings* out) {
    if (out == nullptr) return;
    out->max_newton_iterations = 30;
    out->max_line_search_halvings = 12;
    out->rounding_floor_W_m2 = 1e-3;
    out->max_non_monotone_steps = 4;
    out->max_non_monotone_growth = 100.0;
    out->newton_tolerance_W_m2 = 1e-6;
    out->cg_relative_tolerance = 1e-6;
    out->max_cg_iterations = 2000;
}

int psgb_solve_implicit_transport_device(psgb_planet* planet, double conductance_W_K, const double* source_floor_W_m2,
                                         psgb_device_response response, void* user,
                                         const psgb_transport_settings* settings_in,
                                         const psgb_solve_options* options, const double* latent_W_m2,
                                         double* source_out_W_m2, double* mean_out_K, psgb_transport_result* result,
                                         int memory, void* stream) {
    return guarded([&] {
        require(planet != nullptr && source_floor_W_m2 != nullptr && response != nullptr &&
                    source_out_W_m2 != nullptr && mean_out_K != nullptr,
                "null argument");
        require(memory == PSGB_MEMORY_HOST || memory == PSGB_MEMORY_DEVICE,
                "memory must be PSGB_MEMORY_HOST or PSGB_MEMORY_DEVICE");
        require(std::isfinite(conductance_W_K) && conductance_W_K > 0.0,
                "transport conductance must be finite and positive");
        const psgb_transport_settings settings = checked_settings(settings_in);
        const Setup g = setup(planet);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        DeviceResponse r;
        r.fn = response;
        r.user = user;
        r.n = g.n;
        r.st = st;
        Solver s{planet, g.n, conductance_W_K, g.area, nullptr, r, {}, workspace(planet, g.n), st};
        psgb_solve_options_default(&s.inner);
        if (options != nullptr) s.inner = *options;
        s.inner.tolerance = settings.cg_relative_tolerance;
        s.inner.max_iterations = settings.max_cg_iterations;
        copy_vector(s.w.floor, source_floor_W_m2, g.n, memory, true, st);
        if (latent_W_m2 != nullptr) {
            copy_vector(s.w.latent, latent_W_m2, g.n, memory, true, st);
            s.latent = s.w.latent;
        }
        const psgb_transport_result out = newton(s, settings);
        copy_vector(source_out_W_m2, s.w.source, g.n, memory, false, st);
        copy_vector(mean_out_K, s.w.mean, g.n, memory, false, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        if (result != nullptr) *result = out;
        return PSGB_OK;
    });
}

int psgb_solve_implicit_transport(psgb_planet* planet, double conductance_W_K, const double* source_floor_W_m2,
                                  psgb_transport_response response, void* user,
                                  const psgb_transport_settings* settings_in, const psgb_solve_options* options,
                                  const double* latent_W_m2, double* source_out_W_m2, double* mean_out_K,
                                  psgb_transport_result* result) {
    return guarded([&] {
        require(planet != nullptr && source_floor_W_m2 != nullptr && response != nullptr &&
                    source_out_W_m2 != nullptr && mean_out_K != nullptr,
                "null argument");
        require(std::isfinite(conductance_W_K) && conductance_W_K > 0.0,
                "transport conductance must be finite and positive");
        const psgb_transport_settings settings = checked_settings(settings_in);
        const Setup g = setup(planet);
        cudaStream_t st = nullptr;
        Workspace w = workspace(planet, g.n);
        HostResponse r;
        r.fn = response;
        r.user = user;
        r.n = g.n;
        r.w = &w;
        r.st = st;
        Solver s{planet, g.n, conductance_W_K, g.area, nullptr, r, {}, w, st};
        psgb_solve_options_default(&s.inner);
        if (options != nullptr) s.inner = *options;
        s.inner.tolerance = settings.cg_relative_tolerance;
        s.inner.max_iterations = settings.max_cg_iterations;
        copy_vector(s.w.floor, source_floor_W_m2, g.n, PSGB_MEMORY_HOST, true, st);
        if (latent_W_m2 != nullptr) {
            copy_vector(s.w.latent, latent_W_m2, g.n, PSGB_MEMORY_HOST, true, st);
            s.latent = s.w.latent;
        }
        const psgb_transport_result out = newton(s, settings);
        copy_vector(source_out_W_m2, s.w.source, g.n, PSGB_MEMORY_HOST, false, st);
        copy_vector(mean_out_K, s.w.mean, g.n, PSGB_MEMORY_HOST, false, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        if (result != nullptr) *result = out;
        return PSGB_OK;
    });
}

int psgb_quartic_device_response(void* user, uint64_t cells, const double* source_W_m2, double* mean_K,
                                 double* slope_K_m2_W, void* stream) {
    return guarded([&] {
        const auto* q = static_cast<const psgb_quartic_response*>(user);
        require(q != nullptr && q->b != nullptr && source_W_m2 != nullptr && mean_K != nullptr &&
                    slope_K_m2_W != nullptr,
                "null argument");
        require(q->a > 0.0 && q->radiative > 0.0, "the quartic's coefficients must be positive");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (q->planet == nullptr) {
            k_quartic<<<blocks_of(cells), kThreads, 0, st>>>(static_cast<std::uint32_t>(cells), q->a, q->radiative, q->b,
                                                            q->hold_stride, q->hold_K, nullptr, source_W_m2, mean_K,
                                                            slope_K_m2_W);
            PSGB_CHECK_LAUNCH();
            return PSGB_OK;
        }
        // Per fine cell of an agglomerated planet, then the nodes' area-weighted means.
        require(!q->planet->planet->group_of_cell.empty(), "not an agglomerated planet");
        require(q->scratch != nullptr, "the fine-cell response needs scratch memory");
        psgb::upload_planet(*q->planet->planet);
        const psgb::DevMesh& d = q->planet->planet->dev;
        require(cells == d.n, "cell count does not match the planet");
        const std::size_t fine = d.fine_cells;
        double* fine_mean = q->scratch;
        double* fine_slope = q->scratch + fine;
        k_quartic<<<blocks_of(fine), kThreads, 0, st>>>(static_cast<std::uint32_t>(fine), q->a, q->radiative, q->b,
                                                       q->hold_stride, q->hold_K, d.group_of_cell, source_W_m2,
                                                       fine_mean, fine_slope);
        PSGB_CHECK_LAUNCH();
        psgb::launch_group_mean(d, fine_mean, fine_slope, mean_K, slope_K_m2_W, st);
        PSGB_CHECK_LAUNCH();
        return PSGB_OK;
    });
}

}  // extern "C"
