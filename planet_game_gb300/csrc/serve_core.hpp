// The continuous-batching request loop for implicit heat-transport sub-steps (host logic).
//
// Requests ask for one sub-step of one registered planet: its temperature advances from
// the planet's current state by the implicit step with the request's source term. Planets
// are grouped into lanes by mesh level; a lane holds its planets' batch and states
// resident on the device while admitted. Each lane has a worker thread that works in
// rounds: it takes, for every planet with queued requests, the oldest one, and steps them
// together (the other planets of the lane are masked out). Requests that arrive during a
// round join the lane's next round, while the other lanes' rounds run concurrently.
//
// Admission is bounded by a device-memory budget: a lane with queued requests that is not
// resident reserves its estimated bytes, evicting the least recently used idle lanes
// (resident, not stepping, nothing queued) first, or waits until a lane goes idle. A lane
// that has waited longer than `yield_after_s` makes the resident lanes that stepped since
// it began waiting yield after their running round, so that under memory pressure the
// lanes take turns instead of a busy lane holding the memory for as long as its requests
// keep coming. A lane whose own estimate exceeds the budget fails its requests with
// PSGB_ERR_BUDGET. An evicted lane's states are copied back to the host first, so no
// sub-step is lost.
//
// The device side is behind Backend/Lane (serve.cpp runs them on the GPU through the batch
// entry points; the host tests use a fake), so this file has no CUDA code.
#pragma once

#include "../../include/planetsim_gb300.h"

#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace psgb::serve {

// A registered planet: its step parameters and, while its lane is not resident, its state.
struct PlanetRecord {
    std::uint32_t level = 0;
    std::uint32_t cells = 0;
    double heat_capacity_J_m2_K = 0.0;
    double dt_s = 0.0;
    double conductance_W_K = 0.0;
    std::vector<double> edge_conductance;   // per undirected edge (empty: conductance_W_K)
    std::vector<double> state_K;            // the temperature after the planet's completed requests
    void* device = nullptr;                 // backend data (the GPU backend's planet handle)
};

// One admitted lane: its planets' resident batch and states.
class Lane {
  public:
    virtual ~Lane() = default;
    // Steps the planets with active[i] != 0 (i indexes the lane's planets) from their
    // resident states with sources[i]; writes the new states to results[i] (host, the
    // planet's cells) and keeps them resident; reports[i] per stepped planet. Throws on
    // failure (the round's requests then fail with the mapped status).
    virtual void step(const std::vector<std::uint8_t>& active, const std::vector<const double*>& sources,
                      const std::vector<double*>& results, std::vector<psgb_step_report>& reports) = 0;
    // Copies the resident state of lane planet i to `out` (the planet's cells).
    virtual void read_state(std::size_t i, double* out) = 0;
};

class Backend {
  public:
    virtual ~Backend() = default;
    // Device bytes reserved for a lane of these planets while it is resident.
    virtual std::uint64_t lane_bytes(const std::vector<const PlanetRecord*>& planets) = 0;
    // Makes the lane resident: its planets' batch, and their states taken from state_K.
    // `first_sources`: per planet, the source of its oldest queued request (null: none),
    // the work the lane is admitted for (a backend that tunes its lanes tunes on these).
    virtual std::unique_ptr<Lane> admit(std::uint32_t level, const std::vector<PlanetRecord*>& planets,
                                        const std::vector<const double*>& first_sources) = 0;
    // Called on a lane's worker thread before its first round (the GPU backend selects
    // the device there).
    virtual void thread_start() {}
};

struct Stats {
    std::uint64_t submitted = 0, completed = 0, failed = 0, rounds = 0, evictions = 0, admissions = 0;
    std::uint64_t resident_bytes = 0;
    std::uint32_t resident_lanes = 0, planets = 0;
    double p50_ms = 0.0, p99_ms = 0.0;   // submit-to-done latency of the completed requests
};

// Maps a failure inside a round or an admission onto a PSGB status code.
using ErrorMapper = int (*)(std::exception_ptr error, std::string& message);

class Server {
  public:
    Server(std::unique_ptr<Backend> backend, double budget_bytes, ErrorMapper mapper, double yield_after_s = 0.25);
    ~Server();   // stops the lanes after their current round; queued requests fail
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    std::uint32_t add_planet(PlanetRecord record);
    // Queues a sub-step of `planet` with this source (copied); returns its request id.
    std::uint64_t submit(std::uint32_t planet, const double* source_W_m2);
    // Waits up to timeout_s (negative: no limit) for the request. On completion copies the
    // new temperature (if t_new_K) and the report (if report), forgets the request and
    // returns its status; PSGB_ERR_TIMEOUT if it is still running.
    int wait(std::uint64_t request, double timeout_s, double* t_new_K, psgb_step_report* report,
             std::string& message);
    // The planet's temperature after its completed requests (waits for a running round).
    void state(std::uint32_t planet, double* out);
    Stats stats();
    // Forgets the counts and latencies so far (e.g. after a warm-up); resident lanes stay.
    // Meant for an idle server: a request in flight completes into the new counts.
    void reset_stats();
    std::uint32_t cells(std::uint32_t planet);

  private:
    struct Request {
        std::uint64_t id = 0;
        std::uint32_t planet = 0;
        std::vector<double> source, result;
        psgb_step_report report{};
        int status = -1;
        bool done = false;
        std::string message;
        double submitted_s = 0.0, done_s = 0.0;
    };
    enum class Phase { Absent, Admitting, Resident, Evicting };
    struct LaneState {
        std::uint32_t level = 0;
        std::vector<std::uint32_t> planets;                      // registry ids, in lane order
        std::map<std::uint32_t, std::size_t> index;              // registry id -> lane index
        std::vector<std::deque<std::shared_ptr<Request>>> queue; // per lane planet
        std::unique_ptr<Lane> lane;
        Phase phase = Phase::Absent;
        bool busy = false;        // a round (or a state read) is using the resident lane
        std::uint64_t bytes = 0;  // reserved while resident
        double last_used_s = 0.0;
        double waiting_since_s = -1.0;   // waiting for memory since (negative: not waiting)
        std::condition_variable cv;
        std::thread thread;
        bool has_work() const;
    };

    void run_lane(LaneState* lane);
    bool admit(LaneState* lane, std::unique_lock<std::mutex>& lock);
    void fail_queued(LaneState* lane, int status, const std::string& message);
    void complete(const std::vector<std::shared_ptr<Request>>& round, int status, const std::string& message);
    double now_s() const;
    // True when resident lane `o` must make way for lane `waiter` (waiting long enough, and
    // `o` has stepped since it began waiting).
    bool yields_to(const LaneState* o, const LaneState* waiter, double now) const;
    const LaneState* starving_waiter(const LaneState* o, double now) const;
    void stop_waiting(LaneState* lane);

    std::unique_ptr<Backend> backend_;
    const double budget_;
    ErrorMapper mapper_;
    const double yield_after_s_;
    std::mutex mu_;
    std::condition_variable done_cv_, memory_cv_;
    std::vector<std::unique_ptr<PlanetRecord>> planets_;   // stable addresses for the lanes
    std::map<std::uint32_t, std::unique_ptr<LaneState>> lanes_;   // by mesh level
    std::unordered_map<std::uint64_t, std::shared_ptr<Request>> requests_;
    std::vector<double> latencies_ms_;
    std::uint64_t next_request_ = 1;
    std::uint64_t resident_bytes_ = 0;   // lanes holding device memory (resident, evicting or being built)
    std::uint64_t pending_bytes_ = 0;    // promised to lanes whose victims are still being evicted
    Stats counts_;
    bool stopping_ = false;
    const std::chrono::steady_clock::time_point start_;
};

}  // namespace psgb::serve
