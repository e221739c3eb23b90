// The continuous-batching request loop's host logic (see serve_core.hpp).
#include "serve_core.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace psgb::serve {

bool Server::LaneState::has_work() const {
    for (const auto& q : queue)
        if (!q.empty()) return true;
    return false;
}

Server::Server(std::unique_ptr<Backend> backend, double budget_bytes, ErrorMapper mapper, double yield_after_s)
    : backend_(std::move(backend)),
      budget_(budget_bytes),
      mapper_(mapper),
      yield_after_s_(yield_after_s),
      start_(std::chrono::steady_clock::now()) {
    if (!backend_ || mapper_ == nullptr) throw std::invalid_argument("serve: null backend or error mapper");
    if (!(budget_bytes > 0.0)) throw std::invalid_argument("serve: the memory budget must be positive");
    if (!(yield_after_s >= 0.0)) throw std::invalid_argument("serve: the yield delay must be non-negative");
}

bool Server::yields_to(const LaneState* o, const LaneState* waiter, double now) const {
    return waiter != o && waiter->waiting_since_s >= 0.0 && now - waiter->waiting_since_s >= yield_after_s_ &&
           o->last_used_s >= waiter->waiting_since_s;
}

const Server::LaneState* Server::starving_waiter(const LaneState* o, double now) const {
    for (const auto& [level, w] : lanes_)
        if (yields_to(o, w.get(), now)) return w.get();
    return nullptr;
}

void Server::stop_waiting(LaneState* L) {
    if (L->waiting_since_s < 0.0) return;
    L->waiting_since_s = -1.0;
    for (auto& [level, lane] : lanes_) lane->cv.notify_all();   // lanes that yielded to it resume
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lock(mu_);
        stopping_ = true;
        for (auto& [level, lane] : lanes_) lane->cv.notify_all();
        memory_cv_.notify_all();
        done_cv_.notify_all();
    }
    for (auto& [level, lane] : lanes_)
        if (lane->thread.joinable()) lane->thread.join();
    lanes_.clear();   // the resident lanes' device memory goes before the backend
}

double Server::now_s() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - start_).count();
}

std::uint32_t Server::add_planet(PlanetRecord record) {
    std::lock_guard<std::mutex> lock(mu_);
    if (stopping_) throw std::logic_error("serve: the server is closing");
    if (record.cells == 0 || record.state_K.size() != record.cells)
        throw std::invalid_argument("serve: a planet needs its cell count and initial state");
    if (lanes_.count(record.level) != 0)
        throw std::invalid_argument("serve: register a level's planets before the level's first request");
    planets_.push_back(std::make_unique<PlanetRecord>(std::move(record)));
    return static_cast<std::uint32_t>(planets_.size() - 1);
}

std::uint32_t Server::cells(std::uint32_t planet) {
    std::lock_guard<std::mutex> lock(mu_);
    if (planet >= planets_.size()) throw std::invalid_argument("serve: unknown planet");
    return planets_[planet]->cells;
}

std::uint64_t Server::submit(std::uint32_t planet, const double* source_W_m2) {
    std::lock_guard<std::mutex> lock(mu_);
    if (stopping_) throw std::logic_error("serve: the server is closing");
    if (planet >= planets_.size()) throw std::invalid_argument("serve: unknown planet");
    if (source_W_m2 == nullptr) throw std::invalid_argument("serve: null source");
    const PlanetRecord& rec = *planets_[planet];
    auto& slot = lanes_[rec.level];
    if (!slot) {   // the level's lane: every planet of the level registered so far
        slot = std::make_unique<LaneState>();
        slot->level = rec.level;
        for (std::uint32_t id = 0; id < planets_.size(); ++id) {
            if (planets_[id]->level != rec.level) continue;
            slot->index[id] = slot->planets.size();
            slot->planets.push_back(id);
        }
        slot->queue.resize(slot->planets.size());
        LaneState* raw = slot.get();
        slot->thread = std::thread([this, raw] { run_lane(raw); });
    }
    auto r = std::make_shared<Request>();
    r->id = next_request_++;
    r->planet = planet;
    r->source.assign(source_W_m2, source_W_m2 + rec.cells);
    r->submitted_s = now_s();
    slot->queue[slot->index.at(planet)].push_back(r);
    requests_[r->id] = r;
    ++counts_.submitted;
    slot->cv.notify_all();
    return r->id;
}

int Server::wait(std::uint64_t request, double timeout_s, double* t_new_K, psgb_step_report* report,
                 std::string& message) {
    std::unique_lock<std::mutex> lock(mu_);
    auto it = requests_.find(request);
    if (it == requests_.end()) throw std::invalid_argument("serve: unknown request");
    std::shared_ptr<Request> r = it->second;
    const auto ready = [&] { return r->done; };
    if (timeout_s < 0.0) {
        done_cv_.wait(lock, ready);
    } else if (!done_cv_.wait_for(lock, std::chrono::duration<double>(timeout_s), ready)) {
        return PSGB_ERR_TIMEOUT;
    }
    if (t_new_K != nullptr && r->result.size() == planets_[r->planet]->cells)
        std::copy(r->result.begin(), r->result.end(), t_new_K);
    if (report != nullptr) *report = r->report;
    message = r->message;
    requests_.erase(r->id);
    return r->status;
}

void Server::state(std::uint32_t planet, double* out) {
    std::unique_lock<std::mutex> lock(mu_);
    if (planet >= planets_.size()) throw std::invalid_argument("serve: unknown planet");
    if (out == nullptr) throw std::invalid_argument("serve: null output");
    const PlanetRecord& rec = *planets_[planet];
    auto found = lanes_.find(rec.level);
    if (found == lanes_.end()) {
        std::copy(rec.state_K.begin(), rec.state_K.end(), out);
        return;
    }
    LaneState* L = found->second.get();
    L->cv.wait(lock, [&] { return (L->phase == Phase::Absent || L->phase == Phase::Resident) && !L->busy; });
    if (L->phase == Phase::Absent) {
        std::copy(rec.state_K.begin(), rec.state_K.end(), out);
        return;
    }
    L->busy = true;
    const std::size_t i = L->index.at(planet);
    lock.unlock();
    std::exception_ptr error;
    try {
        L->lane->read_state(i, out);
    } catch (...) {
        error = std::current_exception();
    }
    lock.lock();
    L->busy = false;
    L->cv.notify_all();
    memory_cv_.notify_all();
    if (error) std::rethrow_exception(error);
}

Stats Server::stats() {
    std::lock_guard<std::mutex> lock(mu_);
    Stats s = counts_;
    s.resident_bytes = resident_bytes_;
    s.planets = static_cast<std::uint32_t>(planets_.size());
    for (const auto& [level, lane] : lanes_) s.resident_lanes += lane->phase == Phase::Resident ? 1u : 0u;
    if (!latencies_ms_.empty()) {
        std::vector<double> v = latencies_ms_;
        std::sort(v.begin(), v.end());
        const auto pct = [&](double q) {   // linear interpolation between closest ranks
            const double pos = q * static_cast<double>(v.size() - 1);
            const std::size_t lo = static_cast<std::size_t>(std::floor(pos));
            const std::size_t hi = std::min(lo + 1, v.size() - 1);
            return v[lo] + (pos - static_cast<double>(lo)) * (v[hi] - v[lo]);
        };
        s.p50_ms = pct(0.50);
        s.p99_ms = pct(0.99);
    }
    return s;
}

void Server::reset_stats() {
    std::lock_guard<std::mutex> lock(mu_);
    counts_ = Stats{};
    latencies_ms_.clear();
}

void Server::fail_queued(LaneState* L, int status, const std::string& message) {
    std::vector<std::shared_ptr<Request>> failed;
    for (auto& q : L->queue) {
        while (!q.empty()) {
            failed.push_back(q.front());
            q.pop_front();
        }
    }
    complete(failed, status, message);
}

void Server::complete(const std::vector<std::shared_ptr<Request>>& round, int status, const std::string& message) {
    const double t = now_s();
    for (const auto& r : round) {
        if (!r) continue;
        if (status != PSGB_OK) {   // the round failed: no new temperature
            r->status = status;
            r->message = message;
            r->result.clear();
        } else {
            r->status = r->report.solve.status;
        }
        r->done = true;
        r->done_s = t;
        if (r->status == PSGB_OK) {
            ++counts_.completed;
            latencies_ms_.push_back((r->done_s - r->submitted_s) * 1e3);
        } else {
            ++counts_.failed;
        }
    }
    done_cv_.notify_all();
}

// Called with the lock held by a lane whose phase is Absent and which has queued work.
// Returns true once the lane is resident; false when it must wait and retry, or when its
// queued requests were failed.
bool Server::admit(LaneState* L, std::unique_lock<std::mutex>& lock) {
    std::vector<const PlanetRecord*> crecs;
    std::vector<PlanetRecord*> recs;
    for (std::uint32_t id : L->planets) {
        crecs.push_back(planets_[id].get());
        recs.push_back(planets_[id].get());
    }
    std::uint64_t need = 0;
    try {
        need = backend_->lane_bytes(crecs);
    } catch (...) {
        std::string message;
        const int status = mapper_(std::current_exception(), message);
        stop_waiting(L);
        fail_queued(L, status, message);
        return false;
    }
    if (static_cast<double>(need) > budget_) {
        stop_waiting(L);
        fail_queued(L, PSGB_ERR_BUDGET, "serve: the lane's device memory exceeds the budget");
        return false;
    }
    // idle lanes go first (least recently used first), then lanes yielding to this one;
    // the bytes promised to lanes being admitted right now count as taken
    const double now = now_s();
    std::vector<LaneState*> victims;
    std::uint64_t freed = 0;
    while (static_cast<double>(resident_bytes_ + pending_bytes_ - freed + need) > budget_) {
        LaneState* victim = nullptr;
        bool victim_idle = false;
        for (auto& [level, other] : lanes_) {
            LaneState* o = other.get();
            if (o == L || o->phase != Phase::Resident || o->busy) continue;
            const bool idle = !o->has_work();
            if (!idle && !yields_to(o, L, now)) continue;
            if (std::find(victims.begin(), victims.end(), o) != victims.end()) continue;
            if (victim == nullptr || (idle && !victim_idle) ||
                (idle == victim_idle && o->last_used_s < victim->last_used_s)) {
                victim = o;
                victim_idle = idle;
            }
        }
        if (victim == nullptr) {   // every resident lane is busy: wait for one to go idle or yield
            if (L->waiting_since_s < 0.0) L->waiting_since_s = now;
            memory_cv_.wait_for(lock, std::chrono::duration<double>(std::max(yield_after_s_, 1e-3)));
            return false;
        }
        victims.push_back(victim);
        freed += victim->bytes;
    }
    stop_waiting(L);
    // the requests the lane is admitted for (held, so their sources outlive the unlock;
    // they leave the queue only in this lane's own rounds)
    std::vector<std::shared_ptr<Request>> firsts(L->planets.size());
    std::vector<const double*> first_sources(L->planets.size(), nullptr);
    for (std::size_t i = 0; i < L->planets.size(); ++i) {
        if (L->queue[i].empty()) continue;
        firsts[i] = L->queue[i].front();
        first_sources[i] = firsts[i]->source.data();
    }
    for (LaneState* v : victims) v->phase = Phase::Evicting;
    L->phase = Phase::Admitting;
    // promised before the lock is let go, so that a lane admitted while the victims are
    // evicted sees these bytes as taken (the budget holds at every moment)
    pending_bytes_ += need;
    lock.unlock();
    for (LaneState* v : victims) {
        for (std::size_t i = 0; i < v->planets.size(); ++i) {
            PlanetRecord& rec = *planets_[v->planets[i]];
            try {
                v->lane->read_state(i, rec.state_K.data());
            } catch (...) {
                // a device failure here keeps the state of the lane's last admission
            }
        }
        v->lane.reset();
    }
    lock.lock();
    for (LaneState* v : victims) {
        resident_bytes_ -= v->bytes;
        v->bytes = 0;
        v->phase = Phase::Absent;
        ++counts_.evictions;
        v->cv.notify_all();
    }
    pending_bytes_ -= need;
    resident_bytes_ += need;
    L->bytes = need;
    lock.unlock();
    std::unique_ptr<Lane> made;
    int status = PSGB_OK;
    std::string message;
    try {
        made = backend_->admit(L->level, recs, first_sources);
        if (!made) throw std::logic_error("serve: the backend admitted no lane");
    } catch (...) {
        status = mapper_(std::current_exception(), message);
    }
    lock.lock();
    if (!made) {
        resident_bytes_ -= need;
        L->bytes = 0;
        L->phase = Phase::Absent;
        fail_queued(L, status, message);
        memory_cv_.notify_all();
        return false;
    }
    L->lane = std::move(made);
    L->phase = Phase::Resident;
    L->last_used_s = now_s();
    ++counts_.admissions;
    return true;
}

void Server::run_lane(LaneState* L) {
    try {
        backend_->thread_start();
    } catch (...) {
    }
    std::unique_lock<std::mutex> lock(mu_);
    for (;;) {
        L->cv.wait(lock, [&] {
            return stopping_ || (L->has_work() && !L->busy && (L->phase == Phase::Absent || L->phase == Phase::Resident));
        });
        if (stopping_) {
            fail_queued(L, PSGB_ERR_LOGIC, "serve: the server closed before the request ran");
            return;
        }
        if (L->phase == Phase::Absent) {
            admit(L, lock);
            continue;
        }
        if (starving_waiter(L, now_s()) != nullptr) {   // make way: stay idle until evicted or no longer asked
            memory_cv_.notify_all();
            L->cv.wait_for(lock, std::chrono::duration<double>(std::max(yield_after_s_, 1e-3)));
            continue;
        }
        // one round: the oldest request of every planet with queued work
        const std::size_t n = L->planets.size();
        std::vector<std::shared_ptr<Request>> round(n);
        std::vector<std::uint8_t> active(n, 0);
        std::vector<const double*> sources(n, nullptr);
        std::vector<double*> results(n, nullptr);
        std::vector<psgb_step_report> reports(n);
        for (std::size_t i = 0; i < n; ++i) {
            if (L->queue[i].empty()) continue;
            round[i] = L->queue[i].front();
            L->queue[i].pop_front();
        }
        try {
            for (std::size_t i = 0; i < n; ++i) {
                if (!round[i]) continue;
                round[i]->result.resize(planets_[L->planets[i]]->cells);
                active[i] = 1;
                sources[i] = round[i]->source.data();
                results[i] = round[i]->result.data();
            }
        } catch (...) {
            std::string message;
            const int status = mapper_(std::current_exception(), message);
            complete(round, status, message);
            continue;
        }
        L->busy = true;
        lock.unlock();
        int status = PSGB_OK;
        std::string message;
        try {
            L->lane->step(active, sources, results, reports);
        } catch (...) {
            status = mapper_(std::current_exception(), message);
        }
        lock.lock();
        for (std::size_t i = 0; i < n; ++i)
            if (round[i]) round[i]->report = reports[i];
        complete(round, status, message);
        L->busy = false;
        L->last_used_s = now_s();
        ++counts_.rounds;
        memory_cv_.notify_all();
        L->cv.notify_all();
    }
}

}  // namespace psgb::serve
