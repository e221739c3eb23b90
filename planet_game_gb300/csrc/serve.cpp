// The serving loop's device side and its C ABI (the loop itself: serve_core.cpp).
//
// A resident lane is one psgb_batch of the level's planets, a private non-blocking
// stream, and two device arrays with the planets back to back: their temperatures and a
// staging area for the round's sources. A round copies the active planets' sources in,
// steps them with psgb_batch_transport_step_masked on device arrays (the temperatures
// are both the step's input and its output: the batch takes its inputs in before it
// writes its outputs), and copies their new temperatures out. Solve statuses (not
// converged, breakdown, non-finite) are per request; any other failure fails the round.
#include "capi_internal.hpp"
#include "serve_core.hpp"

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>

namespace psgb::serve {
namespace {

// A failed library call: its status code and message.
struct StatusError : std::runtime_error {
    int code;
    StatusError(int c, const std::string& message) : std::runtime_error(message), code(c) {}
};

void check(int status) {
    if (status != PSGB_OK) throw StatusError(status, psgb_last_error());
}

bool solve_status(int status) {
    return status == PSGB_ERR_NOT_CONVERGED || status == PSGB_ERR_BREAKDOWN || status == PSGB_ERR_NON_FINITE;
}

int map_error(std::exception_ptr error, std::string& message) {
    try {
        std::rethrow_exception(error);
    } catch (const StatusError& e) {
        message = e.what();
        return e.code;
    } catch (...) {
        const int code = psgb::capi::guarded([&]() -> int { std::rethrow_exception(std::current_exception()); });
        message = psgb::capi::g_last_error;
        return code;
    }
}

struct Tunings {
    std::mutex mu;
    std::map<std::uint32_t, psgb_tuning> by_level;
};

class GpuLane final : public Lane {
  public:
    GpuLane(const psgb_server_config& cfg, std::uint32_t level, const std::vector<PlanetRecord*>& planets,
            const std::vector<const double*>& first_sources, Tunings& tunings)
        : options_(cfg.options) {
        try {
            build(cfg, level, planets, first_sources, tunings);
        } catch (...) {
            release();   // a partly built lane frees what it holds
            throw;
        }
    }

    ~GpuLane() override { release(); }

    GpuLane(const GpuLane&) = delete;
    GpuLane& operator=(const GpuLane&) = delete;

    void step(const std::vector<std::uint8_t>& active, const std::vector<const double*>& sources,
              const std::vector<double*>& results, std::vector<psgb_step_report>& reports) override {
        const std::size_t n = cells_.size();
        std::vector<const double*> t0(n), src(n);
        std::vector<double*> t_new(n);
        for (std::size_t i = 0; i < n; ++i) {
            t0[i] = states_ + offset_[i];
            t_new[i] = states_ + offset_[i];
            src[i] = sources_ + offset_[i];
            if (active[i])
                PSGB_CUDA(cudaMemcpyAsync(sources_ + offset_[i], sources[i], cells_[i] * sizeof(double),
                                          cudaMemcpyHostToDevice, stream_));
        }
        const int status = psgb_batch_transport_step_masked(batch_, active.data(), params_.data(), &options_, t0.data(),
                                                            src.data(), t_new.data(), nullptr, reports.data(),
                                                            PSGB_MEMORY_DEVICE, stream_);
        if (status != PSGB_OK && !solve_status(status)) throw StatusError(status, psgb_last_error());
        for (std::size_t i = 0; i < n; ++i)
            if (active[i])
                PSGB_CUDA(cudaMemcpyAsync(results[i], states_ + offset_[i], cells_[i] * sizeof(double),
                                          cudaMemcpyDeviceToHost, stream_));
        PSGB_CUDA(cudaStreamSynchronize(stream_));
    }

    void read_state(std::size_t i, double* out) override {
        PSGB_CUDA(cudaMemcpyAsync(out, states_ + offset_[i], cells_[i] * sizeof(double), cudaMemcpyDeviceToHost,
                                  stream_));
        PSGB_CUDA(cudaStreamSynchronize(stream_));
    }

  private:
    void build(const psgb_server_config& cfg, std::uint32_t level, const std::vector<PlanetRecord*>& planets,
               const std::vector<const double*>& first_sources, Tunings& tunings) {
        const std::size_t n = planets.size();
        std::vector<psgb_planet*> handles(n);
        std::size_t total = 0;
        for (std::size_t i = 0; i < n; ++i) {
            handles[i] = static_cast<psgb_planet*>(planets[i]->device);
            offset_.push_back(total);
            cells_.push_back(planets[i]->cells);
            total += planets[i]->cells;
        }
        PSGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        PSGB_CUDA(cudaMalloc(reinterpret_cast<void**>(&states_), total * sizeof(double)));
        PSGB_CUDA(cudaMalloc(reinterpret_cast<void**>(&sources_), total * sizeof(double)));
        for (std::size_t i = 0; i < n; ++i)
            PSGB_CUDA(cudaMemcpyAsync(states_ + offset_[i], planets[i]->state_K.data(), cells_[i] * sizeof(double),
                                      cudaMemcpyHostToDevice, stream_));
        PSGB_CUDA(cudaMemsetAsync(sources_, 0, total * sizeof(double), stream_));
        // a lane tuned at admission tunes on the requests it was admitted for (zero
        // sources elsewhere: those planets converge at once and do not set the pace)
        for (std::size_t i = 0; i < n && i < first_sources.size(); ++i)
            if (first_sources[i] != nullptr)
                PSGB_CUDA(cudaMemcpyAsync(sources_ + offset_[i], first_sources[i], cells_[i] * sizeof(double),
                                          cudaMemcpyHostToDevice, stream_));
        check(psgb_batch_create(handles.data(), static_cast<std::uint32_t>(n), &batch_));
        params_.resize(n);
        std::vector<const double*> edges(n, nullptr);
        bool any_edges = false;
        for (std::size_t i = 0; i < n; ++i) {
            const PlanetRecord& p = *planets[i];
            params_[i] = psgb_step_params{p.heat_capacity_J_m2_K, p.dt_s, p.conductance_W_K, nullptr, 0};
            if (!p.edge_conductance.empty()) {
                edges[i] = p.edge_conductance.data();
                params_[i].edge_conductance_stored = 1;
                any_edges = true;
            }
        }
        if (any_edges) check(psgb_batch_set_edge_conductance(batch_, edges.data()));
        if (cfg.autotune) {
            bool have = false;
            psgb_tuning tuning{};
            {
                std::lock_guard<std::mutex> lock(tunings.mu);
                auto found = tunings.by_level.find(level);
                if (found != tunings.by_level.end()) {
                    tuning = found->second;
                    have = true;
                }
            }
            if (have) {
                check(psgb_batch_set_tuning(batch_, &tuning));
            } else {
                std::vector<const double*> t0(n), src(n);
                for (std::size_t i = 0; i < n; ++i) {
                    t0[i] = states_ + offset_[i];
                    src[i] = sources_ + offset_[i];
                }
                check(psgb_batch_autotune(batch_, params_.data(), &options_, t0.data(), src.data(), PSGB_MEMORY_DEVICE,
                                          stream_, &tuning));
                std::lock_guard<std::mutex> lock(tunings.mu);
                tunings.by_level.emplace(level, tuning);
            }
        }
        PSGB_CUDA(cudaStreamSynchronize(stream_));
    }

    void release() noexcept {
        if (stream_ != nullptr) cudaStreamSynchronize(stream_);
        if (batch_ != nullptr) psgb_batch_destroy(batch_);
        if (states_ != nullptr) cudaFree(states_);
        if (sources_ != nullptr) cudaFree(sources_);
        if (stream_ != nullptr) cudaStreamDestroy(stream_);
        batch_ = nullptr;
        states_ = sources_ = nullptr;
        stream_ = nullptr;
    }

    psgb_solve_options options_;
    psgb_batch* batch_ = nullptr;
    cudaStream_t stream_ = nullptr;
    double* states_ = nullptr;
    double* sources_ = nullptr;
    std::vector<std::size_t> offset_, cells_;
    std::vector<psgb_step_params> params_;
};

class GpuBackend final : public Backend {
  public:
    explicit GpuBackend(const psgb_server_config& cfg) : cfg_(cfg) {
        if (!(cfg_.bytes_per_cell > 0.0)) cfg_.bytes_per_cell = 700.0;
    }
    ~GpuBackend() override {
        for (psgb_planet* p : planets_) psgb_planet_destroy(p);
    }
    GpuBackend(const GpuBackend&) = delete;
    GpuBackend& operator=(const GpuBackend&) = delete;

    std::uint64_t lane_bytes(const std::vector<const PlanetRecord*>& planets) override {
        double cells = 0.0;
        for (const PlanetRecord* p : planets) cells += p->cells;
        return static_cast<std::uint64_t>(std::ceil(cells * cfg_.bytes_per_cell));
    }
    std::unique_ptr<Lane> admit(std::uint32_t level, const std::vector<PlanetRecord*>& planets,
                                const std::vector<const double*>& first_sources) override {
        return std::make_unique<GpuLane>(cfg_, level, planets, first_sources, tunings_);
    }
    void thread_start() override { PSGB_CUDA(cudaSetDevice(cfg_.device)); }

    // Keeps a planet handle for the server's life (destroyed with the backend).
    void keep(psgb_planet* planet) {
        std::lock_guard<std::mutex> lock(mu_);
        planets_.push_back(planet);
    }

  private:
    psgb_server_config cfg_;
    Tunings tunings_;
    std::mutex mu_;
    std::vector<psgb_planet*> planets_;
};

}  // namespace
}  // namespace psgb::serve

struct psgb_server {
    psgb::serve::GpuBackend* backend = nullptr;   // owned by the server
    std::unique_ptr<psgb::serve::Server> server;
};

using psgb::capi::guarded;

namespace {

void require(bool ok, const char* message) {
    if (!ok) throw std::invalid_argument(message);
}

}  // namespace

extern "C" {

int psgb_server_create(const psgb_server_config* config, psgb_server** out) {
    return guarded([&] {
        require(config != nullptr && out != nullptr, "null argument");
        *out = nullptr;
        require(std::isfinite(config->budget_bytes) && config->budget_bytes > 0.0, "the budget must be positive");
        require(std::isfinite(config->bytes_per_cell), "bytes per cell must be finite");
        require(config->device >= 0, "negative device");
        static_cast<void>(psgb::capi::to_options(&config->options));   // validates the options
        auto backend = std::make_unique<psgb::serve::GpuBackend>(*config);
        auto h = std::make_unique<psgb_server>();
        h->backend = backend.get();
        require(std::isfinite(config->yield_after_s), "the yield delay must be finite");
        const double yield_after = config->yield_after_s > 0.0 ? config->yield_after_s : 0.25;
        h->server = std::make_unique<psgb::serve::Server>(std::move(backend), config->budget_bytes,
                                                          psgb::serve::map_error, yield_after);
        *out = h.release();
        return PSGB_OK;
    });
}

void psgb_server_destroy(psgb_server* server) { delete server; }

int psgb_server_add_planet(psgb_server* server, uint32_t level, double radius_m, const psgb_step_params* params,
                           const double* t0_K, uint32_t* planet_out) {
    return guarded([&] {
        require(server != nullptr && params != nullptr && t0_K != nullptr && planet_out != nullptr, "null argument");
        require(std::isfinite(params->heat_capacity_J_m2_K) && params->heat_capacity_J_m2_K > 0.0 &&
                    std::isfinite(params->dt_s) && params->dt_s > 0.0,
                "heat capacity and time step must be positive");
        require(std::isfinite(params->conductance_W_K) && params->conductance_W_K >= 0.0,
                "conductance must be finite and non-negative");
        require(params->edge_conductance_stored == 0, "pass the planet's edge conductances in params");
        psgb_planet* raw = nullptr;
        const int status = psgb_planet_create(level, radius_m, &raw);
        if (status != PSGB_OK) return psgb::capi::fail(status, psgb_last_error());
        std::unique_ptr<psgb_planet, void (*)(psgb_planet*)> handle(raw, psgb_planet_destroy);
        psgb_planet_info info{};
        if (psgb_planet_info_get(raw, &info) != PSGB_OK) return psgb::capi::fail(PSGB_ERR_LOGIC, psgb_last_error());
        psgb::serve::PlanetRecord rec;
        rec.level = level;
        rec.cells = static_cast<std::uint32_t>(info.cells);
        rec.heat_capacity_J_m2_K = params->heat_capacity_J_m2_K;
        rec.dt_s = params->dt_s;
        rec.conductance_W_K = params->conductance_W_K;
        if (params->edge_conductance != nullptr) {
            rec.edge_conductance.assign(params->edge_conductance, params->edge_conductance + info.edges);
            for (double e : rec.edge_conductance)
                require(std::isfinite(e) && e >= 0.0, "edge conductances must be finite and non-negative");
        }
        rec.state_K.assign(t0_K, t0_K + rec.cells);
        for (double t : rec.state_K) require(std::isfinite(t), "non-finite initial temperature");
        rec.device = raw;
        *planet_out = server->server->add_planet(std::move(rec));
        server->backend->keep(handle.release());
        return PSGB_OK;
    });
}

int psgb_server_submit(psgb_server* server, uint32_t planet, const double* source_W_m2, uint64_t* request_out) {
    return guarded([&] {
        require(server != nullptr && source_W_m2 != nullptr && request_out != nullptr, "null argument");
        const std::uint32_t cells = server->server->cells(planet);
        for (std::uint32_t c = 0; c < cells; ++c) require(std::isfinite(source_W_m2[c]), "non-finite source");
        *request_out = server->server->submit(planet, source_W_m2);
        return PSGB_OK;
    });
}

int psgb_server_wait(psgb_server* server, uint64_t request, double timeout_s, double* t_new_K,
                     psgb_step_report* report) {
    return guarded([&] {
        require(server != nullptr, "null argument");
        std::string message;
        const int status = server->server->wait(request, timeout_s, t_new_K, report, message);
        if (status == PSGB_ERR_TIMEOUT) return psgb::capi::fail(status, "the request is still queued or running");
        if (status != PSGB_OK)
            return psgb::capi::fail(status, message.empty() ? psgb::capi::status_message(status) : message);
        return PSGB_OK;
    });
}

int psgb_server_state(psgb_server* server, uint32_t planet, double* t_K) {
    return guarded([&] {
        require(server != nullptr && t_K != nullptr, "null argument");
        server->server->state(planet, t_K);
        return PSGB_OK;
    });
}

int psgb_server_stats_get(psgb_server* server, psgb_server_stats* out) {
    return guarded([&] {
        require(server != nullptr && out != nullptr, "null argument");
        const psgb::serve::Stats s = server->server->stats();
        *out = psgb_server_stats{s.submitted, s.completed, s.failed, s.rounds, s.evictions, s.admissions,
                                 s.resident_bytes, s.resident_lanes, s.planets, s.p50_ms, s.p99_ms};
        return PSGB_OK;
    });
}

int psgb_server_stats_reset(psgb_server* server) {
    return guarded([&] {
        require(server != nullptr, "null argument");
        server->server->reset_stats();
        return PSGB_OK;
    });
}

}  // extern "C"
