// Stage times of the front end, printed to stderr when the environment
// variable SYMGB_FRONTEND_TIMES is set (no cost otherwise).
#pragma once

#include <chrono>
#include <cstdio>
#include <cstdlib>

namespace symgb {

class StageClock {
public:
    StageClock() : on_(std::getenv("SYMGB_FRONTEND_TIMES") != nullptr), last_(std::chrono::steady_clock::now()) {}
    void mark(const char* stage) {
        if (!on_) return;
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "symgb front end: %-24s %8.3f s\n", stage,
                     std::chrono::duration<double>(now - last_).count());
        last_ = now;
    }

private:
    bool on_;
    std::chrono::steady_clock::time_point last_;
};

}  // namespace symgb
