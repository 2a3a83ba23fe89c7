// Data-parallel loops for the host front end.
#pragma once
#include <cstddef>
#include <functional>

namespace symgb {

// Runs fn(begin, end) over [0, n) in chunks of at least `grain` items on a
// process-wide pool of worker threads (the calling thread takes part) and
// returns when every chunk is done.  Loops of fewer than 2 * grain items, and
// loops started from inside a pool worker, run on the calling thread.  fn must
// not throw.  The pool size is the hardware thread count, or SYMGB_THREADS
// when that environment variable is set (1 = serial).
void parallelFor(std::size_t n, std::size_t grain, const std::function<void(std::size_t, std::size_t)>& fn);

// Threads the pool uses (including the caller).
int frontEndThreads();

}  // namespace symgb
