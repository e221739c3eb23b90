// Launch accounting and opt-in per-kernel timing (see profile.hpp).
#include "profile.hpp"

#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

namespace psgb {
namespace {

std::atomic<std::uint64_t> g_launches[kFamCount];
std::atomic<std::uint64_t> g_graph_kernels{0};
thread_local bool g_capturing = false;

struct Profile {
    std::mutex mu;
    std::atomic<int> family{-1};
    std::vector<cudaEvent_t> start, stop;
    std::size_t used = 0;          // event pairs handed out
    std::uint64_t launches = 0;
    std::uint64_t generation = 0;  // bumped by every profile_begin
} g_profile;

// The event pair a thread's launch_begin handed out, closed by the same thread's
// launch_end: two host threads launching the same family (lanes stepped side by side)
// each time their own launch.
struct PendingSlot {
    std::size_t index = 0;
    std::uint64_t generation = 0;
    bool open = false;
};
thread_local PendingSlot t_pending;

constexpr std::size_t kMaxEvents = 1 << 16;

const char* const kNames[kFamCount] = {"smooth", "residual", "restrict", "prolong", "dense", "krylov_spmv",
                                       "krylov_vector", "refine", "setup", "step", "operator", "column",
                                       "persistent", "smooth_coarse", "residual_coarse", "restrict_coarse",
                                       "prolong_coarse"};

}  // namespace

const char* family_name(int family) { return family >= 0 && family < kFamCount ? kNames[family] : "?"; }

int family_of(const char* name) {
    for (int f = 0; f < kFamCount; ++f)
        if (name != nullptr && std::strcmp(name, kNames[f]) == 0) return f;
    return -1;
}

bool profile_active() { return g_profile.family >= 0; }

namespace {
unsigned long long* g_bytes_counter = nullptr;   // device, allocated by the first profile_begin
}

unsigned long long* profile_bytes_for(int family) {
    return g_profile.family == family ? g_bytes_counter : nullptr;
}

std::uint64_t profile_bytes_exchange() {
    if (g_bytes_counter == nullptr) return 0;
    unsigned long long v = 0;
    cudaMemcpy(&v, g_bytes_counter, sizeof(v), cudaMemcpyDeviceToHost);
    cudaMemset(g_bytes_counter, 0, sizeof(v));
    return v;
}
void set_capturing(bool on) { g_capturing = on; }
void count_graph_kernels(std::uint64_t kernels) { g_graph_kernels.fetch_add(kernels, std::memory_order_relaxed); }

void launch_begin(int family, cudaStream_t st) {
    if (g_capturing) return;
    g_launches[family].fetch_add(1, std::memory_order_relaxed);
    if (g_profile.family != family) return;
    std::lock_guard<std::mutex> lock(g_profile.mu);
    if (g_profile.family != family || g_profile.used >= kMaxEvents) return;
    if (g_profile.used == g_profile.start.size()) {
        cudaEvent_t a, b;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return;
        g_profile.start.push_back(a);
        g_profile.stop.push_back(b);
    }
    t_pending = PendingSlot{g_profile.used, g_profile.generation, true};
    cudaEventRecord(g_profile.start[g_profile.used], st);
    ++g_profile.used;
}

void launch_end(int family, cudaStream_t st) {
    if (g_capturing || g_profile.family != family || !t_pending.open) return;
    std::lock_guard<std::mutex> lock(g_profile.mu);
    t_pending.open = false;
    if (t_pending.generation != g_profile.generation || g_profile.family != family) return;
    cudaEventRecord(g_profile.stop[t_pending.index], st);
    ++g_profile.launches;
}

std::uint64_t launches_total() {
    std::uint64_t s = g_graph_kernels.load(std::memory_order_relaxed);
    for (auto& c : g_launches) s += c.load(std::memory_order_relaxed);
    return s;
}

std::uint64_t launches_of(int family) { return g_launches[family].load(std::memory_order_relaxed); }

bool profile_begin(int family) {
    if (family < 0 || family >= kFamCount) return false;
    if (g_bytes_counter == nullptr) {
        if (cudaMalloc(&g_bytes_counter, sizeof(unsigned long long)) != cudaSuccess) return false;
    }
    cudaMemset(g_bytes_counter, 0, sizeof(unsigned long long));
    std::lock_guard<std::mutex> lock(g_profile.mu);
    g_profile.family = family;
    g_profile.used = 0;
    g_profile.launches = 0;
    ++g_profile.generation;
    return true;
}

bool profile_end(double* total_ms, std::uint64_t* launches) {
    std::lock_guard<std::mutex> lock(g_profile.mu);
    if (g_profile.family < 0) return false;
    double sum = 0.0;
    // every slot handed out was closed by its launch_end (launches complete before a
    // profile ends: the caller synchronises its steps first)
    for (std::size_t i = 0; i < g_profile.used; ++i) {
        cudaEventSynchronize(g_profile.stop[i]);
        float ms = 0.0F;
        if (cudaEventElapsedTime(&ms, g_profile.start[i], g_profile.stop[i]) == cudaSuccess) sum += ms;
    }
    *total_ms = sum;
    *launches = g_profile.launches;
    g_profile.family = -1;
    ++g_profile.generation;
    return true;
}

}  // namespace psgb
