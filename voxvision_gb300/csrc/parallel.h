/* parallel.h -- the library's host thread pool for one loop. */
#ifndef VOX_PARALLEL_H
#define VOX_PARALLEL_H

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

/* Runs f(i) for i in [0, n) on up to all host threads, indices dealt
 * dynamically.  Threads that cannot be started leave their share to the
 * others (the calling thread always takes part).  The first exception thrown
 * by f stops the loop and is rethrown in the calling thread once every thread
 * has ended: no exception ends a pool thread, which would end the process. */
template <typename F>
void parallel_for(size_t n, F f)
{
    size_t nt = std::min<size_t>(n, std::max(1u, std::thread::hardware_concurrency()));
    if (nt <= 1) {
        for (size_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::exception_ptr err;
    std::mutex err_mu;
    auto run = [&]() {
        try {
            for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
        } catch (...) {
            std::lock_guard<std::mutex> g(err_mu);
            if (!err) err = std::current_exception();
            next.store(n);
        }
    };
    std::vector<std::thread> pool;
    try {
        pool.reserve(nt - 1);
        for (size_t t = 1; t < nt; t++) pool.emplace_back(run);
    } catch (...) {
        // fewer threads: the rest do the whole loop
    }
    run();
    for (auto &th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

#endif
