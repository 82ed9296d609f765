#pragma once

// Timing harness with the project's semantics (src/bench.hpp:1-44): every operation hands its
// upload / compute / download phases to Bench::run(), which runs them `warmup` times untimed and
// then `runs` times with CUDA events around each phase on the legacy default stream. Setup
// (allocation, plans) happens before run() and stays out of every number.

#include <functional>

struct BenchConfig {
    int warmup = 0;
    int runs = 1;
};

struct PhaseTime {
    double mean_ms = 0.0;
    double std_ms = 0.0;  // sample standard deviation (n - 1); zero for one run
};

struct BenchResult {
    PhaseTime h2d;
    PhaseTime kernel;
    PhaseTime d2h;
};

class Bench {
public:
    explicit Bench(BenchConfig config) : config_(config) {}

    void run(const std::function<void()>& upload, const std::function<void()>& compute,
             const std::function<void()>& download);

    const BenchConfig& config() const { return config_; }
    const BenchResult& result() const { return result_; }

private:
    BenchConfig config_;
    BenchResult result_;
};
