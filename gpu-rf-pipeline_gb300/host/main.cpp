// rfgpu: the command-line front end for this library's filtering path, with the gpu-rf-pipeline
// tool's grammar for the operations it covers (src/main.cpp:1-13):
//
//   rfgpu fir        --in X.cf32 --taps H.f32 --out Y.cf32 [--impl NAME] [--block B]
//   rfgpu channelize --in X.cf32 --taps H.f32 --channels M --out Z.cf32 [--impl NAME]
//                    [--output complex|magnitude]   (magnitude: |z| as float32, fused)
//   rfgpu magnitude  --in X.cf32 --out MAG.f32
//   rfgpu stream     --in X.cf32 --taps H.f32 --out Y.cf32 [--impl NAME] [--chunk N]
//                    [--depth D] [--memory copy|registered|zero-copy] [--rate HZ]
//   rfgpu info
//   (every X input may be a SigMF recording, NAME.sigmf-meta or NAME.sigmf-data, in cf32_le,
//    ci16_le or ci8; fir and channelize: [--bench N [--warmup W]] prints phase timings as JSON; stream: the
//    wall-clock time of whole streamed passes, with the throughput against the sample rate)
//
// Exit status: 0 on success, 1 on a runtime error (file, CUDA, cuFFT), 2 on a usage error.
#include "bench.hpp"
#include "check.hpp"
#include "io.hpp"
#include "ops.hpp"
#include "stream.hpp"

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

struct UsageError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

template <class Fn>
std::string impl_names(const std::vector<Impl<Fn>>& impls, const char* sep)
{
    std::string s;
    for (const Impl<Fn>& impl : impls) {
        if (!s.empty()) {
            s += sep;
        }
        s += impl.name;
    }
    return s;
}

template <class Fn>
void print_impls(const char* op, const std::vector<Impl<Fn>>& impls)
{
    for (std::size_t i = 0; i < impls.size(); ++i) {
        std::fprintf(stderr, "  %-10s --impl %-12s %s%s\n", op, impls[i].name, impls[i].summary,
                     i == 0 ? " (default)" : "");
    }
}

void print_usage()
{
    std::fprintf(stderr,
                 "usage:\n"
                 "  rfgpu fir        --in X.cf32 --taps H.f32 --out OUT.cf32 [--impl NAME] "
                 "[--block B]\n"
                 "  rfgpu channelize --in X.cf32 --taps H.f32 --channels M --out OUT.cf32 "
                 "[--impl NAME]\n"
                 "                  [--output complex|magnitude]  magnitude: |z| per channel as "
                 "float32\n"
                 "  rfgpu magnitude  --in X.cf32 --out OUT.f32\n"
                 "  rfgpu stream     --in X.cf32 --taps H.f32 --out OUT.cf32 [--impl NAME] "
                 "[--chunk N]\n"
                 "                  [--depth D] [--memory copy|registered|zero-copy] [--rate HZ]\n"
                 "                  FIR in chunks through a ring of D pinned buffers and CUDA streams\n"
                 "  rfgpu info       GPU, CUDA versions and implementations as JSON\n"
                 "\n"
                 "Every .cf32 input may also be a SigMF recording (NAME.sigmf-meta or "
                 "NAME.sigmf-data)\n"
                 "in cf32_le, ci16_le or ci8; fir converts integer recordings on the GPU.\n"
                 "\n"
                 "benchmark options (fir, channelize, magnitude, stream):\n"
                 "  --bench N      time N runs with CUDA events and print the result as JSON\n"
                 "  --warmup W     untimed runs before measuring (default 3, needs --bench)\n"
                 "\n"
                 "implementations:\n");
    print_impls("fir", fir_impls());
    print_impls("channelize", channelize_impls());
}

// "--flag value" pairs of one subcommand, each flag at most once and from an allowed set.
class Args {
public:
    Args(int argc, char** argv, const std::set<std::string>& allowed)
    {
        for (int i = 2; i < argc; i += 2) {
            const std::string flag = argv[i];
            if (allowed.count(flag) == 0) {
                throw UsageError("unknown option '" + flag + "' for " + argv[1]);
            }
            if (i + 1 >= argc) {
                throw UsageError("option " + flag + " needs a value");
            }
            if (!values_.emplace(flag, argv[i + 1]).second) {
                throw UsageError("option " + flag + " given twice");
            }
        }
    }

    bool has(const std::string& flag) const { return values_.count(flag) != 0; }

    const std::string& required(const std::string& flag) const
    {
        const auto it = values_.find(flag);
        if (it == values_.end()) {
            throw UsageError("missing required option " + flag);
        }
        return it->second;
    }

    std::string optional(const std::string& flag, const std::string& fallback) const
    {
        const auto it = values_.find(flag);
        return it == values_.end() ? fallback : it->second;
    }

    int integer(const std::string& flag, int fallback, int minimum) const
    {
        const auto it = values_.find(flag);
        if (it == values_.end()) {
            return fallback;
        }
        char* end = nullptr;
        const long v = std::strtol(it->second.c_str(), &end, 10);
        if (end == it->second.c_str() || *end != '\0' || v < minimum || v > INT_MAX) {
            throw UsageError(flag + " needs an integer of at least " + std::to_string(minimum) +
                             ", got '" + it->second + "'");
        }
        return static_cast<int>(v);
    }

private:
    std::map<std::string, std::string> values_;
};

template <class Fn>
const Impl<Fn>& find_impl(const std::vector<Impl<Fn>>& impls, const Args& args, const char* op)
{
    const std::string name = args.optional("--impl", impls.front().name);
    for (const Impl<Fn>& impl : impls) {
        if (name == impl.name) {
            return impl;
        }
    }
    throw UsageError("unknown --impl '" + name + "' for " + op + " (available: " +
                     impl_names(impls, ", ") + ")");
}

BenchConfig bench_config(const Args& args)
{
    BenchConfig config;
    if (args.has("--bench")) {
        config.runs = args.integer("--bench", 1, 1);
        config.warmup = args.integer("--warmup", 3, 0);
    } else if (args.has("--warmup")) {
        throw UsageError("--warmup needs --bench");
    }
    return config;
}

void require_int_range(std::size_t count, const std::string& what)
{
    if (count > static_cast<std::size_t>(INT_MAX)) {
        throw std::runtime_error(what + " has " + std::to_string(count) +
                                 " elements, more than the supported " + std::to_string(INT_MAX));
    }
}

std::string gpu_name()
{
    int device = 0;
    CUDA_CHECK(cudaGetDevice(&device));
    cudaDeviceProp prop{};
    CUDA_CHECK(cudaGetDeviceProperties(&prop, device));
    return prop.name;
}

void report(const Args& args, const char* op, const char* impl, std::size_t num_in,
            std::size_t num_out, const Bench& bench);

void finish(const Args& args, const char* op, const char* impl, std::size_t num_in,
            const std::vector<cf32>& out, const Bench& bench)
{
    write_cf32(args.required("--out"), out);
    report(args, op, impl, num_in, out.size(), bench);
}

void finish_f32(const Args& args, const char* op, const char* impl, std::size_t num_in,
                const std::vector<float>& out, const Bench& bench)
{
    write_f32(args.required("--out"), out);
    report(args, op, impl, num_in, out.size(), bench);
}

void report(const Args& args, const char* op, const char* impl, std::size_t num_in,
            std::size_t num_out, const Bench& bench)
{
    const std::string& path = args.required("--out");
    if (!args.has("--bench")) {
        std::printf("%s[%s]: %zu samples in, %zu out -> %s\n", op, impl, num_in, num_out,
                    path.c_str());
        return;
    }
    const BenchResult& r = bench.result();
    std::printf("{\"op\": \"%s\", \"impl\": \"%s\", \"gpu\": \"%s\", \"num_in\": %zu, "
                "\"num_out\": %zu, \"runs\": %d, \"warmup\": %d, "
                "\"h2d_ms\": {\"mean\": %.6f, \"std\": %.6f}, "
                "\"kernel_ms\": {\"mean\": %.6f, \"std\": %.6f}, "
                "\"d2h_ms\": {\"mean\": %.6f, \"std\": %.6f}}\n",
                op, impl, gpu_name().c_str(), num_in, num_out, bench.config().runs,
                bench.config().warmup, r.h2d.mean_ms, r.h2d.std_ms, r.kernel.mean_ms,
                r.kernel.std_ms, r.d2h.mean_ms, r.d2h.std_ms);
}

int run_fir(int argc, char** argv)
{
    const Args args(argc, argv,
                    {"--in", "--taps", "--out", "--impl", "--block", "--bench", "--warmup"});
    args.required("--out");
    const Impl<FirFn>& impl = find_impl(fir_impls(), args, "fir");
    const int block = args.integer("--block", kDefaultFirBlock, 32);
    if (block % 32 != 0 || block > 1024) {
        throw UsageError("--block needs a multiple of 32 up to 1024, got " +
                         std::to_string(block));
    }
    Bench bench(bench_config(args));
    // Integer recordings go to the device as stored and are converted there (a half or a
    // quarter of the upload); the results are those of converting on the host first.
    StoredSamples stored = read_stored(args.required("--in"));
    const std::vector<float> taps = read_f32(args.required("--taps"));
    if (taps.empty()) {
        throw std::runtime_error(args.required("--taps") + ": no taps");
    }
    require_int_range(stored.count, "fir input");
    require_int_range(taps.size(), "tap array");
    const std::size_t num_in = stored.count;
    std::vector<cf32> y;
    if (num_in > 0 && stored.format != SampleFormat::Cf32) {
        y = fir_stored(impl.name, stored, taps, block, bench);
    } else if (num_in > 0) {
        const std::vector<cf32> x = to_cf32(stored);
        stored.bytes = std::vector<std::uint8_t>();
        y = impl.fn(x, taps, block, bench);
    }
    finish(args, "fir", impl.name, num_in, y, bench);
    return 0;
}

int run_channelize(int argc, char** argv)
{
    const Args args(argc, argv, {"--in", "--taps", "--channels", "--out", "--impl", "--output",
                                 "--bench", "--warmup"});
    args.required("--out");
    if (!args.has("--channels")) {
        throw UsageError("missing required option --channels");
    }
    const int channels = args.integer("--channels", 0, 1);
    const Impl<ChanFn>& impl = find_impl(channelize_impls(), args, "channelize");
    const std::string output = args.optional("--output", "complex");
    if (output != "complex" && output != "magnitude") {
        throw UsageError("unknown --output '" + output + "' (available: complex, magnitude)");
    }
    Bench bench(bench_config(args));
    StoredSamples stored = read_stored(args.required("--in"));
    const std::vector<float> taps = read_f32(args.required("--taps"));
    if (taps.empty()) {
        throw std::runtime_error(args.required("--taps") + ": no taps");
    }
    require_int_range(stored.count + static_cast<std::size_t>(channels),
                      "padded channelizer input");
    require_int_range(taps.size(), "tap array");
    if (stored.format != SampleFormat::Cf32) {
        // Integer recordings go to the device as stored and are converted there.
        std::vector<cf32> z;
        std::vector<float> mag;
        channelize_stored(impl.name, stored, taps, channels, output == "magnitude", z, mag, bench);
        if (output == "magnitude") {
            finish_f32(args, "channelize", impl.name, stored.count, mag, bench);
        } else {
            finish(args, "channelize", impl.name, stored.count, z, bench);
        }
        return 0;
    }
    const std::vector<cf32> x = to_cf32(stored);
    stored.bytes = std::vector<std::uint8_t>();
    if (output == "magnitude") {
        finish_f32(args, "channelize", impl.name, x.size(),
                   channelize_magnitude(impl.name, x, taps, channels, bench), bench);
        return 0;
    }
    finish(args, "channelize", impl.name, x.size(), impl.fn(x, taps, channels, bench), bench);
    return 0;
}

// |x| of every sample (src/main.cpp:255-267).
int run_magnitude(int argc, char** argv)
{
    const Args args(argc, argv, {"--in", "--out", "--bench", "--warmup"});
    args.required("--out");
    Bench bench(bench_config(args));
    const std::vector<cf32> x = read_cf32(args.required("--in"));
    require_int_range(x.size(), "magnitude input");
    const std::vector<float> mag = x.empty() ? std::vector<float>() : magnitude_cuda(x, bench);
    finish_f32(args, "magnitude", "elementwise", x.size(), mag, bench);
    return 0;
}

// Streamed FIR (stream.hpp). Without --bench: one pass, written to --out. With --bench N: W
// untimed passes, then N timed ones, reported as JSON with the throughput against --rate (or
// the input's sample rate from its metadata).
int run_stream(int argc, char** argv)
{
    const Args args(argc, argv, {"--in", "--taps", "--out", "--impl", "--chunk", "--depth",
                                 "--memory", "--rate", "--bench", "--warmup"});
    args.required("--out");
    StreamConfig config;
    const std::string impl = args.optional("--impl", "tiled");
    if (!parse_fir_impl(impl.c_str(), config.impl)) {
        throw UsageError("unknown --impl '" + impl + "' for stream (available: " +
                         impl_names(fir_impls(), ", ") + ")");
    }
    const std::string memory = args.optional("--memory", "copy");
    if (!parse_stream_memory(memory, config.memory)) {
        throw UsageError("unknown --memory '" + memory +
                         "' (available: copy, registered, zero-copy)");
    }
    config.chunk = args.integer("--chunk", config.chunk, 1);
    config.depth = args.integer("--depth", config.depth, 1);
    const BenchConfig bench = bench_config(args);
    // Integer recordings stream as stored (half or a quarter of the bytes over the host link)
    // and are converted on the GPU, with the bits of streaming the converted samples.
    const StoredSamples x = read_stored(args.required("--in"));
    const std::vector<float> taps = read_f32(args.required("--taps"));
    if (taps.empty()) {
        throw std::runtime_error(args.required("--taps") + ": no taps");
    }
    require_int_range(x.count, "stream input");
    require_int_range(static_cast<std::size_t>(config.chunk) + taps.size(), "chunk with history");
    double rate = sample_rate(args.required("--in"));
    if (args.has("--rate")) {
        rate = std::stod(args.required("--rate"));
    }
    std::vector<double> times;
    std::vector<cf32> y;
    StreamTiming timing;
    const int passes = args.has("--bench") ? bench.warmup + bench.runs : 1;
    for (int i = 0; i < passes; ++i) {
        y = fir_stream(x, taps, config, timing);
        if (i >= passes - bench.runs) {
            times.push_back(timing.total_ms);
        }
    }
    write_cf32(args.required("--out"), y);
    if (!args.has("--bench")) {
        std::printf("stream[%s]: %zu samples in %d chunks of %d, depth %d -> %s\n", impl.c_str(),
                    x.count, timing.chunks, config.chunk, config.depth,
                    args.required("--out").c_str());
        return 0;
    }
    double mean = 0.0;
    for (double t : times) {
        mean += t / static_cast<double>(times.size());
    }
    double var = 0.0;
    for (double t : times) {
        var += (t - mean) * (t - mean);
    }
    const double std_ms =
        times.size() > 1 ? std::sqrt(var / static_cast<double>(times.size() - 1)) : 0.0;
    const double msps = mean > 0 ? static_cast<double>(x.count) / (mean * 1e3) : 0.0;
    std::printf("{\"op\": \"stream\", \"impl\": \"%s\", \"memory\": \"%s\", \"gpu\": \"%s\", "
                "\"num_in\": %zu, \"chunk\": %d, \"depth\": %d, \"chunks\": %d, \"runs\": %d, "
                "\"warmup\": %d, \"total_ms\": {\"mean\": %.6f, \"std\": %.6f}, \"msps\": %.3f, "
                "\"sample_rate\": %.1f, \"realtime_factor\": %.3f}\n",
                impl.c_str(), memory.c_str(), gpu_name().c_str(), x.count, config.chunk,
                config.depth, timing.chunks, bench.runs, bench.warmup, mean, std_ms, msps, rate,
                rate > 0 ? msps * 1e6 / rate : 0.0);
    return 0;
}

std::string version_string(int packed)
{
    return std::to_string(packed / 1000) + "." + std::to_string((packed % 1000) / 10);
}

int run_info(int argc, char** argv)
{
    const Args args(argc, argv, {});
    int device = 0;
    CUDA_CHECK(cudaGetDevice(&device));
    cudaDeviceProp prop{};
    CUDA_CHECK(cudaGetDeviceProperties(&prop, device));
    int runtime = 0;
    int driver = 0;
    CUDA_CHECK(cudaRuntimeGetVersion(&runtime));
    CUDA_CHECK(cudaDriverGetVersion(&driver));
    std::printf("{\"gpu\": \"%s\", \"compute_capability\": \"%d.%d\", \"memory_mb\": %zu, "
                "\"sms\": %d, \"cuda_runtime\": \"%s\", \"cuda_driver\": \"%s\", "
                "\"library\": \"%s\", "
                "\"impls\": {\"fir\": [\"%s\"], \"channelize\": [\"%s\"], "
                "\"magnitude\": [\"elementwise\"]}}\n",
                prop.name, prop.major, prop.minor, prop.totalGlobalMem / (1024 * 1024),
                prop.multiProcessorCount, version_string(runtime).c_str(),
                version_string(driver).c_str(), rfx_version(),
                impl_names(fir_impls(), "\", \"").c_str(),
                impl_names(channelize_impls(), "\", \"").c_str());
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        const std::string op = argc > 1 ? argv[1] : "";
        if (op == "fir") return run_fir(argc, argv);
        if (op == "channelize") return run_channelize(argc, argv);
        if (op == "stream") return run_stream(argc, argv);
        if (op == "magnitude") return run_magnitude(argc, argv);
        if (op == "info") return run_info(argc, argv);
        if (op == "--help" || op == "-h" || op == "help") {
            print_usage();
            return 0;
        }
        throw UsageError(op.empty() ? "missing subcommand" : "unknown subcommand '" + op + "'");
    } catch (const UsageError& e) {
        std::fprintf(stderr, "rfgpu: %s\n\n", e.what());
        print_usage();
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "rfgpu: %s\n", e.what());
        return 1;
    }
}
