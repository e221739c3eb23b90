// A minimal fork-join loop over host cores for the mesh and hierarchy builders.
// Each index is processed independently, so results never depend on the number
// of threads; the first exception thrown by any worker is rethrown to the caller.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace psgb {

inline unsigned host_threads() {
    if (const char* env = std::getenv("PSGB_HOST_THREADS")) {
        const int n = std::atoi(env);
        if (n > 0) return static_cast<unsigned>(n);
    }
    const unsigned n = std::thread::hardware_concurrency();
    return n == 0 ? 1u : std::min(n, 64u);
}

template <typename F>
void parallel_for(std::size_t count, F&& body) {
    const unsigned threads = static_cast<unsigned>(
        std::min<std::size_t>(host_threads(), std::max<std::size_t>(1, count / 2048)));
    if (threads <= 1) {
        for (std::size_t i = 0; i < count; ++i) body(i);
        return;
    }
    std::exception_ptr error;
    std::mutex guard;
    std::vector<std::thread> pool;
    pool.reserve(threads);
    const std::size_t chunk = (count + threads - 1) / threads;
    for (unsigned t = 0; t < threads; ++t) {
        const std::size_t begin = t * chunk;
        const std::size_t end = std::min(count, begin + chunk);
        if (begin >= end) break;
        pool.emplace_back([&, begin, end] {
            try {
                for (std::size_t i = begin; i < end; ++i) body(i);
            } catch (...) {
                std::lock_guard<std::mutex> lock(guard);
                if (!error) error = std::current_exception();
            }
        });
    }
    for (auto& th : pool) th.join();
    if (error) std::rethrow_exception(error);
}

}  // namespace psgb
