// Host check of the serving loop's device side (serve.cpp) without a GPU: the CUDA runtime
// calls and the library entry points it uses are replaced by host stand-ins (device
// memory is host memory; the "batch step" is t_new = t0 + dt/C * source, taking every
// input in before writing any output, as the batch does), and the C entry points
// psgb_server_* are driven as a caller would. Checks the lanes' layout of states and
// sources, the stored per-edge conductances, tuning once per level and reuse after
// eviction, states surviving eviction, per-request solve statuses, failed rounds, and
// that destroying the server frees every planet, batch, stream and allocation.
// Prints OK or the first failed check.
#include "../../include/planetsim_gb300.h"
#include "capi_internal.hpp"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace {

int failures = 0;
#define CHECK(cond)                                                            \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);      \
            ++failures;                                                        \
        }                                                                      \
    } while (0)

std::atomic<int> live_planets{0}, live_batches{0}, live_streams{0}, live_allocs{0};
std::atomic<int> autotunes{0}, set_tunings{0}, steps{0}, bad_calls{0};
thread_local std::string stub_error;

struct FakePlanet {
    std::uint32_t level;
    std::uint64_t cells, edges;
};
struct FakeBatch {
    std::vector<FakePlanet*> planets;
    std::vector<std::vector<double>> edges;
};

FakePlanet* fp(const psgb_planet* p) { return reinterpret_cast<FakePlanet*>(const_cast<psgb_planet*>(p)); }
FakeBatch* fb(psgb_batch* b) { return reinterpret_cast<FakeBatch*>(b); }

}  // namespace

// ---- stand-ins for the CUDA runtime -------------------------------------------------------
extern "C" {
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "stand-in error"; }
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned int) {
    *s = reinterpret_cast<cudaStream_t>(new int(0));
    ++live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
    delete reinterpret_cast<int*>(s);
    --live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::malloc(n);
    ++live_allocs;
    return cudaSuccess;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    --live_allocs;
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t n, cudaMemcpyKind, cudaStream_t) {
    std::memcpy(dst, src, n);
    return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t) {
    std::memset(p, v, n);
    return cudaSuccess;
}

// ---- stand-ins for the library entry points the serving loop calls ----------------------
const char* psgb_last_error(void) { return stub_error.c_str(); }
int psgb_planet_create(uint32_t level, double radius_m, psgb_planet** out) {
    if (!(radius_m > 0.0)) {
        stub_error = "radius";
        return PSGB_ERR_INVALID_ARGUMENT;
    }
    const std::uint64_t q = std::uint64_t(1) << (2 * level);
    *out = reinterpret_cast<psgb_planet*>(new FakePlanet{level, 10 * q + 2, 30 * q});
    ++live_planets;
    return PSGB_OK;
}
void psgb_planet_destroy(psgb_planet* p) {
    delete fp(p);
    --live_planets;
}
int psgb_planet_info_get(const psgb_planet* p, psgb_planet_info* out) {
    std::memset(out, 0, sizeof(*out));
    out->cells = fp(p)->cells;
    out->edges = fp(p)->edges;
    return PSGB_OK;
}
int psgb_batch_create(psgb_planet* const* planets, uint32_t count, psgb_batch** out) {
    auto* b = new FakeBatch;
    for (uint32_t i = 0; i < count; ++i) b->planets.push_back(fp(planets[i]));
    b->edges.resize(count);
    *out = reinterpret_cast<psgb_batch*>(b);
    ++live_batches;
    return PSGB_OK;
}
void psgb_batch_destroy(psgb_batch* b) {
    delete fb(b);
    --live_batches;
}
int psgb_batch_set_edge_conductance(psgb_batch* b, const double* const* e) {
    FakeBatch& B = *fb(b);
    for (std::size_t i = 0; i < B.planets.size(); ++i)
        B.edges[i] = e[i] == nullptr ? std::vector<double>{} : std::vector<double>(e[i], e[i] + B.planets[i]->edges);
    return PSGB_OK;
}
int psgb_batch_autotune(psgb_batch*, const psgb_step_params*, const psgb_solve_options*, const double* const* t0,
                        const double* const* src, int memory, void*, psgb_tuning* out) {
    if (memory != PSGB_MEMORY_DEVICE || t0 == nullptr || src == nullptr) ++bad_calls;
    ++autotunes;
    std::memset(out, 0, sizeof(*out));
    out->levels = 7;   // a marker the reapplied tuning must carry
    return PSGB_OK;
}
int psgb_batch_set_tuning(psgb_batch*, const psgb_tuning* t) {
    if (t == nullptr || t->levels != 7) ++bad_calls;
    ++set_tunings;
    return PSGB_OK;
}
// heat capacity 13: the step fails outright; 17: the solve does not converge (the iterate
// is still written, as the batch does)
int psgb_batch_transport_step_masked(psgb_batch* b, const uint8_t* active, const psgb_step_params* params,
                                     const psgb_solve_options*, const double* const* t0, const double* const* src,
                                     double* const* t_new, double* const* transport, psgb_step_report* reports,
                                     int memory, void*) {
    FakeBatch& B = *fb(b);
    if (memory != PSGB_MEMORY_DEVICE || transport != nullptr) ++bad_calls;
    ++steps;
    std::vector<std::vector<double>> in(B.planets.size());
    for (std::size_t i = 0; i < B.planets.size(); ++i) {
        if (!active[i]) continue;
        if (params[i].heat_capacity_J_m2_K == 13.0) {
            stub_error = "stand-in device failure";
            return PSGB_ERR_CUDA;
        }
        if ((params[i].edge_conductance_stored != 0) != !B.edges[i].empty() || params[i].edge_conductance != nullptr)
            ++bad_calls;
        in[i].assign(t0[i], t0[i] + B.planets[i]->cells);   // every input in before any output
    }
    int worst = PSGB_OK;
    for (std::size_t i = 0; i < B.planets.size(); ++i) {
        reports[i] = psgb_step_report{};
        if (!active[i]) continue;
        const double s = params[i].dt_s / params[i].heat_capacity_J_m2_K;
        const double edge_mark = B.edges[i].empty() ? 0.0 : B.edges[i][0];
        for (std::uint64_t c = 0; c < B.planets[i]->cells; ++c) t_new[i][c] = in[i][c] + s * src[i][c] + edge_mark;
        reports[i].solve.iterations = 5;
        reports[i].solve.status = params[i].heat_capacity_J_m2_K == 17.0 ? PSGB_ERR_NOT_CONVERGED : PSGB_OK;
        if (reports[i].solve.status != PSGB_OK) worst = reports[i].solve.status;
    }
    if (worst != PSGB_OK) stub_error = "not converged";
    return worst;
}
}  // extern "C"

// ---- stand-ins for the C ABI's shared helpers ----------------------------------------------
namespace psgb::capi {
thread_local std::string g_last_error;
int fail(int code, const std::string& message) {
    g_last_error = message;
    return code;
}
const char* status_message(int) { return "stand-in status"; }
psgb::SolveOptions to_options(const psgb_solve_options*) { return psgb::SolveOptions{}; }
}  // namespace psgb::capi

namespace {

psgb_server* make_server(double budget, double bytes_per_cell) {
    psgb_server_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.budget_bytes = budget;
    cfg.bytes_per_cell = bytes_per_cell;
    cfg.autotune = 1;
    cfg.yield_after_s = 0.01;
    psgb_server* s = nullptr;
    CHECK(psgb_server_create(&cfg, &s) == PSGB_OK && s != nullptr);
    return s;
}

std::uint32_t add(psgb_server* s, std::uint32_t level, double C, double dt, double t0, const double* edges) {
    const std::uint64_t cells = 10 * (std::uint64_t(1) << (2 * level)) + 2;
    std::vector<double> t(cells, t0);
    psgb_step_params p{C, dt, 5.0, edges, 0};
    std::uint32_t id = 0;
    CHECK(psgb_server_add_planet(s, level, 6.0e6, &p, t.data(), &id) == PSGB_OK);
    return id;
}

double step(psgb_server* s, std::uint32_t planet, std::uint64_t cells, double source, int want = PSGB_OK) {
    std::vector<double> src(cells, source), out(cells, -1.0);
    std::uint64_t r = 0;
    CHECK(psgb_server_submit(s, planet, src.data(), &r) == PSGB_OK);
    psgb_step_report rep{};
    const int st = psgb_server_wait(s, r, 10.0, out.data(), &rep);
    CHECK(st == want);
    if (want == PSGB_OK || want == PSGB_ERR_NOT_CONVERGED) CHECK(rep.solve.iterations == 5 && out[cells - 1] == out[0]);
    return out[0];
}

void lanes_layout_edges_tuning() {
    psgb_server* s = make_server(1e12, 0.0);
    std::vector<double> edges(30 * 4, 0.25);   // level 1: 120 undirected edges
    const std::uint32_t a = add(s, 1, 2.0, 1.0, 100.0, nullptr);        // s = 0.5
    const std::uint32_t b = add(s, 1, 4.0, 1.0, 200.0, edges.data());   // s = 0.25, +0.25 per step
    const std::uint32_t c = add(s, 2, 1.0, 1.0, 300.0, nullptr);        // s = 1
    for (int k = 1; k <= 3; ++k) {
        CHECK(step(s, a, 42, 2.0) == 100.0 + k * 1.0);
        CHECK(step(s, b, 42, 2.0) == 200.0 + k * 0.75);
        CHECK(step(s, c, 162, 2.0) == 300.0 + k * 2.0);
    }
    std::vector<double> now(42);
    CHECK(psgb_server_state(s, b, now.data()) == PSGB_OK && now[41] == 202.25);
    psgb_server_stats st{};
    CHECK(psgb_server_stats_get(s, &st) == PSGB_OK);
    CHECK(st.completed == 9 && st.failed == 0 && st.resident_lanes == 2 && st.admissions == 2 && st.planets == 3);
    CHECK(autotunes.load() == 2 && set_tunings.load() == 0);
    psgb_server_destroy(s);
}

void eviction_keeps_states_and_tuning() {
    const int tunes0 = autotunes.load();
    // 16 bytes per cell and 2 x 42 + 162 cells: room for one lane at a time
    psgb_server* s = make_server(16.0 * 170, 16.0);
    const std::uint32_t a = add(s, 1, 1.0, 1.0, 10.0, nullptr);
    const std::uint32_t c = add(s, 2, 1.0, 1.0, 20.0, nullptr);
    CHECK(step(s, a, 42, 1.0) == 11.0);
    CHECK(step(s, c, 162, 1.0) == 21.0);   // level 1 goes, its state copied back
    std::vector<double> now(42);
    CHECK(psgb_server_state(s, a, now.data()) == PSGB_OK && now[0] == 11.0);
    CHECK(step(s, a, 42, 1.0) == 12.0);    // back with its state and its tuning
    CHECK(step(s, c, 162, 1.0) == 22.0);
    psgb_server_stats st{};
    CHECK(psgb_server_stats_get(s, &st) == PSGB_OK && st.evictions == 3 && st.resident_lanes == 1);
    CHECK(autotunes.load() - tunes0 == 2 && set_tunings.load() == 2);
    psgb_server_destroy(s);
}

void statuses() {
    psgb_server* s = make_server(1e12, 0.0);
    const std::uint32_t good = add(s, 1, 1.0, 1.0, 0.0, nullptr);
    const std::uint32_t slow = add(s, 2, 17.0, 17.0, 0.0, nullptr);   // s = 1, not converged
    const std::uint32_t bad = add(s, 3, 13.0, 13.0, 0.0, nullptr);    // the step fails
    CHECK(step(s, slow, 162, 3.0, PSGB_ERR_NOT_CONVERGED) == 3.0);     // the iterate still comes back
    CHECK(step(s, bad, 642, 3.0, PSGB_ERR_CUDA) == -1.0);
    CHECK(psgb::capi::g_last_error == "stand-in device failure");   // what psgb_last_error() returns
    CHECK(step(s, good, 42, 3.0) == 3.0);
    std::vector<double> now(642);
    CHECK(psgb_server_state(s, bad, now.data()) == PSGB_OK && now[0] == 0.0);   // a failed round keeps the state
    std::uint64_t r = 0;
    std::vector<double> src(42, 1.0);
    src[3] = NAN;
    CHECK(psgb_server_submit(s, good, src.data(), &r) == PSGB_ERR_INVALID_ARGUMENT);
    psgb_server_destroy(s);
}

}  // namespace

int main() {
    lanes_layout_edges_tuning();
    eviction_keeps_states_and_tuning();
    statuses();
    CHECK(bad_calls.load() == 0);
    CHECK(live_planets.load() == 0 && live_batches.load() == 0 && live_streams.load() == 0 && live_allocs.load() == 0);
    if (failures == 0) std::printf("OK\n");
    return failures == 0 ? 0 : 1;
}
