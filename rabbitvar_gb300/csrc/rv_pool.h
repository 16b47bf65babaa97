// A process-wide pool of host worker threads for the data-parallel host
// stages (record text, the tumor/normal classification, the -k 1 realigner,
// batch preparation).  The threads start on first use and are reused, so a
// parallel section costs a wake-up, not thread creation.
#pragma once
#include <cstdint>
#include <functional>

namespace rv {

// Runs fn(i) for every i in [0, n) on the pool and the calling thread;
// returns when all are done.  Rethrows the first exception fn threw.  Runs
// inline when called from inside a parallel section.
void parallel_for(int64_t n, const std::function<void(int64_t)> &fn);

// Threads a parallel section uses (workers + caller).
int pool_threads();

// fn(chunk, begin, end) over [0, n) cut into at most pool_threads() chunks of
// at least min_per_chunk items; returns the number of chunks.
int64_t parallel_chunks(int64_t n, int64_t min_per_chunk, const std::function<void(int64_t, int64_t, int64_t)> &fn);
inline int64_t chunks_for(int64_t n, int64_t min_per_chunk) {
    int64_t c = n / (min_per_chunk > 0 ? min_per_chunk : 1);
    int64_t t = pool_threads();
    c = c < t ? c : t;
    return c > 0 ? c : 1;
}

}  // namespace rv
