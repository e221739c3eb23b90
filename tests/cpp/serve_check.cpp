// Host check of the serving loop (serve_core.cpp) with a fake device backend: a lane's
// "step" is t_new = t + dt/C * source on host arrays, after a short sleep, so rounds take
// time and requests pile up behind them. Prints OK or the first failed check.
#include "serve_core.hpp"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

using namespace psgb::serve;

namespace {

int failures = 0;
#define CHECK(cond)                                                            \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);      \
            ++failures;                                                        \
        }                                                                      \
    } while (0)

struct Counters {
    std::atomic<int> lanes_alive{0}, admissions{0}, rounds{0}, max_concurrent{0}, running{0};
    std::atomic<int> fail_level{-1};          // a step of this level throws
    std::atomic<int> fail_admit_level{-1};    // admission of this level throws
    std::atomic<int> max_round_size{0};
    std::atomic<int> admitted_with_work{0};
};

class FakeLane final : public Lane {
  public:
    FakeLane(Counters& c, std::uint32_t level, const std::vector<PlanetRecord*>& planets) : c_(c), level_(level) {
        for (const PlanetRecord* p : planets) {
            state_.push_back(p->state_K);
            scale_.push_back(p->dt_s / p->heat_capacity_J_m2_K);
        }
        ++c_.lanes_alive;
    }
    ~FakeLane() override { --c_.lanes_alive; }
    void step(const std::vector<std::uint8_t>& active, const std::vector<const double*>& sources,
              const std::vector<double*>& results, std::vector<psgb_step_report>& reports) override {
        const int now = ++c_.running;
        int seen = c_.max_concurrent.load();
        while (now > seen && !c_.max_concurrent.compare_exchange_weak(seen, now)) {
        }
        std::this_thread::sleep_for(std::chrono::milliseconds(3));
        --c_.running;
        if (static_cast<int>(level_) == c_.fail_level.load()) throw std::runtime_error("device step failed");
        int size = 0;
        for (std::size_t i = 0; i < active.size(); ++i) {
            if (!active[i]) continue;
            ++size;
            for (std::size_t k = 0; k < state_[i].size(); ++k) state_[i][k] += scale_[i] * sources[i][k];
            std::copy(state_[i].begin(), state_[i].end(), results[i]);
            reports[i] = psgb_step_report{};
            reports[i].solve.status = PSGB_OK;
            reports[i].solve.iterations = 7;
        }
        int big = c_.max_round_size.load();
        while (size > big && !c_.max_round_size.compare_exchange_weak(big, size)) {
        }
        ++c_.rounds;
    }
    void read_state(std::size_t i, double* out) override { std::copy(state_[i].begin(), state_[i].end(), out); }

  private:
    Counters& c_;
    std::uint32_t level_;
    std::vector<std::vector<double>> state_;
    std::vector<double> scale_;
};

class FakeBackend final : public Backend {
  public:
    FakeBackend(Counters& c, std::uint64_t bytes_per_cell) : c_(c), per_cell_(bytes_per_cell) {}
    std::uint64_t lane_bytes(const std::vector<const PlanetRecord*>& planets) override {
        std::uint64_t cells = 0;
        for (const PlanetRecord* p : planets) cells += p->cells;
        return cells * per_cell_;
    }
    std::unique_ptr<Lane> admit(std::uint32_t level, const std::vector<PlanetRecord*>& planets,
                                const std::vector<const double*>& first_sources) override {
        if (static_cast<int>(level) == c_.fail_admit_level.load()) throw std::invalid_argument("cannot build the lane");
        ++c_.admissions;
        // a lane is admitted for queued work: some planet's oldest source comes along
        bool any = false;
        for (const double* s : first_sources) any = any || s != nullptr;
        if (any && first_sources.size() == planets.size()) ++c_.admitted_with_work;
        return std::make_unique<FakeLane>(c_, level, planets);
    }

  private:
    Counters& c_;
    std::uint64_t per_cell_;
};

int map_error(std::exception_ptr error, std::string& message) {
    try {
        std::rethrow_exception(error);
    } catch (const std::invalid_argument& e) {
        message = e.what();
        return PSGB_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        message = e.what();
        return PSGB_ERR_CUDA;
    }
}

PlanetRecord planet(std::uint32_t level, std::uint32_t cells, double t0) {
    PlanetRecord p;
    p.level = level;
    p.cells = cells;
    p.heat_capacity_J_m2_K = 4.0;
    p.dt_s = 2.0;   // dt/C = 0.5
    p.conductance_W_K = 1.0;
    p.state_K.assign(cells, t0);
    return p;
}

// Three levels of planets; every request's source is 1 + k/100 on planet-local request k;
// each planet's temperature is t0 + 0.5 * the sum of its sources so far.
void continuous_batching_and_order() {
    Counters c;
    Server s(std::make_unique<FakeBackend>(c, 10), 1e12, map_error);
    std::vector<std::uint32_t> ids;
    std::vector<std::uint32_t> cells;
    for (std::uint32_t level : {4u, 5u, 6u})
        for (int k = 0; k < 3; ++k) {
            cells.push_back(8 + level);
            ids.push_back(s.add_planet(planet(level, 8 + level, 250.0 + level)));
        }
    const int per_planet = 12;
    std::vector<std::vector<std::uint64_t>> reqs(ids.size());
    for (int k = 0; k < per_planet; ++k)
        for (std::size_t p = 0; p < ids.size(); ++p) {
            std::vector<double> src(cells[p], 1.0 + k / 100.0);
            reqs[p].push_back(s.submit(ids[p], src.data()));
        }
    bool adding_late_refused = false;
    try {
        s.add_planet(planet(4, 12, 1.0));
    } catch (const std::invalid_argument&) {
        adding_late_refused = true;
    }
    CHECK(adding_late_refused);
    for (std::size_t p = 0; p < ids.size(); ++p) {
        double expect = 250.0 + (p < 3 ? 4 : p < 6 ? 5 : 6);
        for (int k = 0; k < per_planet; ++k) {
            std::vector<double> out(cells[p], -1.0);
            psgb_step_report rep{};
            std::string msg;
            const int st = s.wait(reqs[p][k], 10.0, out.data(), &rep, msg);
            CHECK(st == PSGB_OK);
            expect += 0.5 * (1.0 + k / 100.0);
            CHECK(std::abs(out[0] - expect) < 1e-12 && std::abs(out.back() - expect) < 1e-12);
            CHECK(rep.solve.iterations == 7);
        }
        std::vector<double> now(cells[p]);
        s.state(ids[p], now.data());
        CHECK(std::abs(now[0] - expect) < 1e-12);
    }
    const Stats st = s.stats();
    CHECK(st.submitted == ids.size() * per_planet && st.completed == st.submitted && st.failed == 0);
    CHECK(st.admissions == 3 && st.evictions == 0 && st.resident_lanes == 3);
    CHECK(c.admitted_with_work.load() == 3);     // each lane admitted with its first requests' sources
    CHECK(st.rounds < st.submitted);                 // requests of several planets shared rounds
    CHECK(c.max_round_size.load() == 3);             // a round steps every planet of its level with work
    CHECK(c.max_concurrent.load() >= 2);             // lanes stepped side by side
    CHECK(st.p99_ms >= st.p50_ms && st.p50_ms > 0.0);
    s.reset_stats();
    const Stats zero = s.stats();
    CHECK(zero.submitted == 0 && zero.completed == 0 && zero.p50_ms == 0.0 && zero.resident_lanes == 3);
    std::string msg;
    bool unknown_refused = false;
    try {
        s.wait(reqs[0][0], 0.0, nullptr, nullptr, msg);   // already waited on
    } catch (const std::invalid_argument&) {
        unknown_refused = true;
    }
    CHECK(unknown_refused);
}

// A budget for two of three lanes: the least recently used idle lane goes, its states
// come back with it; a lane larger than the budget fails its requests.
void budget_eviction_and_refusal() {
    Counters c;
    Server s(std::make_unique<FakeBackend>(c, 100), 2 * 2 * 10 * 100 + 50, map_error);   // two lanes of 2x10 cells
    const std::uint32_t a0 = s.add_planet(planet(4, 10, 100.0)), a1 = s.add_planet(planet(4, 10, 100.0));
    const std::uint32_t b0 = s.add_planet(planet(5, 10, 200.0)), b1 = s.add_planet(planet(5, 10, 200.0));
    const std::uint32_t c0 = s.add_planet(planet(6, 10, 300.0)), c1 = s.add_planet(planet(6, 10, 300.0));
    const std::uint32_t big = s.add_planet(planet(7, 100, 1.0));
    std::vector<double> one(10, 1.0);
    std::string msg;
    const auto run = [&](std::uint32_t p) {
        std::vector<double> out(10);
        const std::uint64_t r = s.submit(p, one.data());
        CHECK(s.wait(r, 10.0, out.data(), nullptr, msg) == PSGB_OK);
        return out[0];
    };
    CHECK(run(a0) == 100.5);
    CHECK(run(b0) == 200.5);
    CHECK(s.stats().resident_lanes == 2 && s.stats().evictions == 0);
    CHECK(run(c0) == 300.5);   // level 4 (least recently used) goes
    Stats st = s.stats();
    CHECK(st.evictions == 1 && st.resident_lanes == 2 && c.lanes_alive.load() == 2);
    CHECK(static_cast<double>(st.resident_bytes) <= 2 * 2 * 10 * 100 + 50);
    std::vector<double> now(10);
    s.state(a0, now.data());   // from the host copy taken at eviction
    CHECK(now[0] == 100.5);
    CHECK(run(a0) == 101.0);   // back, with its state: level 5 goes now
    CHECK(run(a1) == 100.5);
    s.state(b0, now.data());
    CHECK(now[0] == 200.5);
    CHECK(run(b1) == 200.5 && run(c1) == 300.5);
    st = s.stats();
    CHECK(st.evictions >= 3 && st.failed == 0);
    std::vector<double> big_src(100, 1.0);
    const std::uint64_t r = s.submit(big, big_src.data());
    CHECK(s.wait(r, 10.0, nullptr, nullptr, msg) == PSGB_ERR_BUDGET);
    CHECK(s.stats().failed == 1);
}

// A failing step fails its round's requests and leaves the planet's state; a failing
// admission fails the lane's queued requests; the server keeps serving the others.
void failures_are_reported() {
    Counters c;
    c.fail_level = 5;
    c.fail_admit_level = 6;
    Server s(std::make_unique<FakeBackend>(c, 1), 1e9, map_error);
    const std::uint32_t a = s.add_planet(planet(4, 4, 10.0));
    const std::uint32_t b = s.add_planet(planet(5, 4, 20.0));
    const std::uint32_t d = s.add_planet(planet(6, 4, 30.0));
    std::vector<double> src(4, 2.0), out(4);
    std::string msg;
    const std::uint64_t rb = s.submit(b, src.data());
    const std::uint64_t rd = s.submit(d, src.data());
    const std::uint64_t ra = s.submit(a, src.data());
    CHECK(s.wait(rb, 10.0, out.data(), nullptr, msg) == PSGB_ERR_CUDA && msg == "device step failed");
    CHECK(s.wait(rd, 10.0, out.data(), nullptr, msg) == PSGB_ERR_INVALID_ARGUMENT && msg == "cannot build the lane");
    CHECK(s.wait(ra, 10.0, out.data(), nullptr, msg) == PSGB_OK && out[0] == 11.0);
    s.state(b, out.data());
    CHECK(out[0] == 20.0);
    const Stats st = s.stats();
    CHECK(st.failed == 2 && st.completed == 1);
}

// A wait that runs out returns PSGB_ERR_TIMEOUT and the request stays; closing the server
// with queued requests fails them instead of hanging.
void timeouts_and_close() {
    Counters c;
    auto s = std::make_unique<Server>(std::make_unique<FakeBackend>(c, 1), 1e9, map_error);
    const std::uint32_t a = s->add_planet(planet(4, 4, 10.0));
    std::vector<double> src(4, 2.0), out(4);
    std::string msg;
    std::vector<std::uint64_t> reqs;
    for (int k = 0; k < 50; ++k) reqs.push_back(s->submit(a, src.data()));   // 50 rounds of 3 ms
    CHECK(s->wait(reqs.back(), 0.0, out.data(), nullptr, msg) == PSGB_ERR_TIMEOUT);
    CHECK(s->wait(reqs.front(), 10.0, out.data(), nullptr, msg) == PSGB_OK && out[0] == 11.0);
    s.reset();   // returns after the running round; the rest fail, nothing hangs
    CHECK(c.lanes_alive.load() == 0);
    bool bad_budget = false;
    try {
        Server bad(std::make_unique<FakeBackend>(c, 1), 0.0, map_error);
    } catch (const std::invalid_argument&) {
        bad_budget = true;
    }
    CHECK(bad_budget);
}

// Four producer threads submit to their own planets of four levels under a budget for two
// lanes: lanes come and go while requests arrive; every request still sees its planet's
// earlier requests, in order.
void concurrent_producers_under_a_tight_budget() {
    Counters c;
    Server s(std::make_unique<FakeBackend>(c, 10), 2 * 3 * 16 * 10 + 5, map_error);   // two lanes of 3 x 16 cells
    std::vector<std::uint32_t> ids;
    for (std::uint32_t level : {3u, 4u, 5u, 6u})
        for (int k = 0; k < 3; ++k) ids.push_back(s.add_planet(planet(level, 16, 100.0 * level)));
    const int per_planet = 20;
    std::vector<std::vector<std::uint64_t>> reqs(ids.size());
    std::vector<std::thread> producers;
    for (int t = 0; t < 4; ++t) {
        producers.emplace_back([&, t] {
            for (int k = 0; k < per_planet; ++k)
                for (std::size_t p = static_cast<std::size_t>(t); p < ids.size(); p += 4) {
                    std::vector<double> src(16, 1.0 + k + p);
                    reqs[p].push_back(s.submit(ids[p], src.data()));
                    if ((k + p) % 5 == 0) std::this_thread::sleep_for(std::chrono::microseconds(300));
                }
        });
    }
    for (auto& th : producers) th.join();
    for (std::size_t p = 0; p < ids.size(); ++p) {
        double expect = 100.0 * (3 + p / 3);
        for (int k = 0; k < per_planet; ++k) {
            std::vector<double> out(16);
            std::string msg;
            CHECK(s.wait(reqs[p][k], 30.0, out.data(), nullptr, msg) == PSGB_OK);
            expect += 0.5 * (1.0 + k + p);
            CHECK(out[7] == expect);
        }
        std::vector<double> now(16);
        s.state(ids[p], now.data());
        CHECK(now[0] == expect);
    }
    const Stats st = s.stats();
    CHECK(st.completed == ids.size() * per_planet && st.failed == 0);
    CHECK(st.evictions > 0 && st.resident_lanes <= 2);
    CHECK(static_cast<double>(st.resident_bytes) <= 2 * 3 * 16 * 10 + 5);
}

// A budget for one lane and two busy levels: past the yield delay the resident lane makes
// way after its round, so the lanes take turns (with their states) instead of the second
// waiting until the first has drained its queue.
void lanes_take_turns_under_pressure() {
    Counters c;
    Server s(std::make_unique<FakeBackend>(c, 1), 8 + 4, map_error, 0.010);   // one lane of 8 cells
    const std::uint32_t a = s.add_planet(planet(4, 8, 10.0));
    const std::uint32_t b = s.add_planet(planet(5, 8, 20.0));
    const int n = 40;   // 40 rounds of 3 ms per lane
    std::vector<double> one(8, 1.0);
    std::vector<std::uint64_t> ra, rb;
    for (int k = 0; k < n; ++k) ra.push_back(s.submit(a, one.data()));
    std::this_thread::sleep_for(std::chrono::milliseconds(2));   // a is resident and busy
    for (int k = 0; k < n; ++k) rb.push_back(s.submit(b, one.data()));
    std::string msg;
    std::vector<double> out(8);
    CHECK(s.wait(rb.front(), 30.0, out.data(), nullptr, msg) == PSGB_OK && out[0] == 20.5);
    // b's first request finished while a still had work queued
    CHECK(s.wait(ra.back(), 0.0, nullptr, nullptr, msg) == PSGB_ERR_TIMEOUT);
    for (int k = 0; k < n; ++k) {
        CHECK(s.wait(ra[k], 30.0, out.data(), nullptr, msg) == PSGB_OK && out[3] == 10.0 + 0.5 * (k + 1));
        if (k > 0) CHECK(s.wait(rb[k], 30.0, out.data(), nullptr, msg) == PSGB_OK && out[3] == 20.0 + 0.5 * (k + 1));
    }
    const Stats st = s.stats();
    CHECK(st.evictions >= 2 && st.failed == 0 && st.completed == 2 * n);
    CHECK(static_cast<double>(st.resident_bytes) <= 12.0 && c.lanes_alive.load() == 1);
}

}  // namespace

int main() {
    continuous_batching_and_order();
    budget_eviction_and_refusal();
    failures_are_reported();
    timeouts_and_close();
    concurrent_producers_under_a_tight_budget();
    lanes_take_turns_under_pressure();
    if (failures == 0) std::printf("OK\n");
    return failures == 0 ? 0 : 1;
}
