#include "bench.hpp"

#include "check.hpp"

#include <cmath>
#include <vector>

namespace {

struct Event {
    cudaEvent_t e{};
    Event() { CUDA_CHECK(cudaEventCreate(&e)); }
    ~Event() { cudaEventDestroy(e); }
    Event(const Event&) = delete;
    Event& operator=(const Event&) = delete;
};

PhaseTime summarize(const std::vector<double>& v)
{
    PhaseTime t;
    if (v.empty()) {
        return t;
    }
    double s = 0.0;
    for (double d : v) {
        s += d;
    }
    t.mean_ms = s / static_cast<double>(v.size());
    if (v.size() > 1) {
        double q = 0.0;
        for (double d : v) {
            q += (d - t.mean_ms) * (d - t.mean_ms);
        }
        t.std_ms = std::sqrt(q / static_cast<double>(v.size() - 1));
    }
    return t;
}

double elapsed(const Event& a, const Event& b)
{
    float ms = 0.0f;
    CUDA_CHECK(cudaEventElapsedTime(&ms, a.e, b.e));
    return ms;
}

}  // namespace

void Bench::run(const std::function<void()>& upload, const std::function<void()>& compute,
                const std::function<void()>& download)
{
    for (int i = 0; i < config_.warmup; ++i) {
        upload();
        compute();
        download();
    }
    Event start, uploaded, computed, downloaded;
    std::vector<double> h2d, kernel, d2h;
    for (int i = 0; i < config_.runs; ++i) {
        CUDA_CHECK(cudaEventRecord(start.e));
        upload();
        CUDA_CHECK(cudaEventRecord(uploaded.e));
        compute();
        CUDA_CHECK(cudaEventRecord(computed.e));
        download();
        CUDA_CHECK(cudaEventRecord(downloaded.e));
        CUDA_CHECK(cudaEventSynchronize(downloaded.e));
        h2d.push_back(elapsed(start, uploaded));
        kernel.push_back(elapsed(uploaded, computed));
        d2h.push_back(elapsed(computed, downloaded));
    }
    result_.h2d = summarize(h2d);
    result_.kernel = summarize(kernel);
    result_.d2h = summarize(d2h);
}
