// rfgpu: the command-line front end of this library's filtering path. Its interface — the
// subcommands, their flags, the JSON reports and the exit codes — is the gpu-rf-pipeline tool's
// for the operations it covers (src/main.cpp:1-13), because that tool's tests drive it:
//
//   rfgpu fir        --in X --taps H.f32 --out Y.cf32 [--impl NAME] [--block B]
//   rfgpu channelize --in X --taps H.f32 --channels M --out Z [--impl NAME]
//                    [--output complex|magnitude]
//   rfgpu magnitude  --in X --out MAG.f32
//   rfgpu stream     --in X --taps H.f32 --out Y.cf32 [--impl NAME] [--chunk N] [--depth D]
//                    [--memory copy|registered|zero-copy] [--rate HZ]
//   rfgpu info
//
// X is a .cf32 file or a SigMF recording (either file of the pair) in cf32_le, ci16_le or ci8.
// fir, channelize, magnitude and stream take [--bench N [--warmup W]].
// Exit status: 0 success, 1 runtime error (file, CUDA, cuFFT), 2 usage error.
//
// Structure: every subcommand is a row of a table (its flags with their value kinds, bounds and
// choices, and its handler). The whole command line is checked against the row before any file
// is opened, so a usage error never leaves a partial output behind; the usage text is printed
// from the same table.
#include "bench.hpp"
#include "check.hpp"
#include "io.hpp"
#include "ops.hpp"
#include "stream.hpp"

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

struct UsageError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// --- the option grammar ----------------------------------------------------------------------

enum class Kind {
    Path,   // any text
    Count,  // an integer in [lo, hi], a multiple of `step`
    Real,   // a finite number
    Word,   // one of choices()
};

struct Flag {
    const char* name;
    Kind kind;
    const char* meta;  // placeholder in the usage text
    bool required;
    long lo;
    long hi;
    long step;
    std::vector<std::string> (*choices)();
    const char* needs;  // another flag this one is only valid with, or nullptr
};

Flag path_flag(const char* name, const char* meta, bool required)
{
    return {name, Kind::Path, meta, required, 0, 0, 1, nullptr, nullptr};
}

Flag count_flag(const char* name, const char* meta, long lo, long hi = INT_MAX, long step = 1,
                bool required = false, const char* needs = nullptr)
{
    return {name, Kind::Count, meta, required, lo, hi, step, nullptr, needs};
}

Flag word_flag(const char* name, const char* meta, std::vector<std::string> (*choices)())
{
    return {name, Kind::Word, meta, false, 0, 0, 1, choices, nullptr};
}

Flag real_flag(const char* name, const char* meta)
{
    return {name, Kind::Real, meta, false, 0, 0, 1, nullptr, nullptr};
}

template <class Fn>
std::vector<std::string> names_of(const std::vector<Impl<Fn>>& table)
{
    std::vector<std::string> out;
    for (const Impl<Fn>& row : table) {
        out.emplace_back(row.name);
    }
    return out;
}

std::vector<std::string> fir_names() { return names_of(fir_impls()); }
std::vector<std::string> chan_names() { return names_of(channelize_impls()); }
std::vector<std::string> output_names() { return {"complex", "magnitude"}; }
std::vector<std::string> memory_names() { return {"copy", "registered", "zero-copy"}; }

std::string joined(const std::vector<std::string>& items, const std::string& glue)
{
    std::string s;
    for (std::size_t i = 0; i < items.size(); ++i) {
        s += (i ? glue : std::string()) + items[i];
    }
    return s;
}

// The validated options of one command line.
class Options {
public:
    bool given(const char* flag) const { return text_.count(flag) != 0; }
    const std::string& text(const char* flag) const { return text_.at(flag); }
    std::string text_or(const char* flag, const std::string& fallback) const
    {
        return given(flag) ? text(flag) : fallback;
    }
    int count_or(const char* flag, int fallback) const
    {
        return given(flag) ? static_cast<int>(std::strtol(text(flag).c_str(), nullptr, 10))
                           : fallback;
    }
    double real(const char* flag) const { return std::strtod(text(flag).c_str(), nullptr); }

    // Bench settings: --bench N timed runs after --warmup W (default 3) untimed ones.
    BenchConfig bench() const
    {
        BenchConfig c;
        if (given("--bench")) {
            c.runs = count_or("--bench", 1);
            c.warmup = count_or("--warmup", 3);
        }
        return c;
    }

    std::map<std::string, std::string> text_;
};

void check_value(const std::string& command, const Flag& f, const std::string& v)
{
    switch (f.kind) {
    case Kind::Path:
        return;
    case Kind::Count: {
        errno = 0;
        char* end = nullptr;
        const long n = std::strtol(v.c_str(), &end, 10);
        const bool number = !v.empty() && *end == '\0' && errno == 0;
        if (!number || n < f.lo || n > f.hi || n % f.step != 0) {
            std::string want = "an integer >= " + std::to_string(f.lo);
            if (f.hi != INT_MAX) {
                want += " and <= " + std::to_string(f.hi);
            }
            if (f.step != 1) {
                want += ", a multiple of " + std::to_string(f.step);
            }
            throw UsageError(command + " " + f.name + " '" + v + "': expected " + want);
        }
        return;
    }
    case Kind::Real: {
        char* end = nullptr;
        const double x = std::strtod(v.c_str(), &end);
        if (v.empty() || *end != '\0' || !std::isfinite(x)) {
            throw UsageError(command + " " + f.name + " '" + v + "': expected a number");
        }
        return;
    }
    case Kind::Word: {
        const std::vector<std::string> ok = f.choices();
        if (std::find(ok.begin(), ok.end(), v) == ok.end()) {
            throw UsageError(command + " " + f.name + " '" + v + "' is not one of: " +
                             joined(ok, ", "));
        }
        return;
    }
    }
}

Options parse(const std::string& command, const std::vector<Flag>& flags,
              const std::vector<std::string>& words)
{
    Options o;
    for (std::size_t i = 0; i < words.size(); i += 2) {
        const std::string& name = words[i];
        const auto f = std::find_if(flags.begin(), flags.end(),
                                    [&](const Flag& g) { return name == g.name; });
        if (f == flags.end()) {
            throw UsageError(command + " has no option '" + name + "'");
        }
        if (i + 1 == words.size()) {
            throw UsageError(command + " " + name + " is missing its value");
        }
        if (o.given(f->name)) {
            throw UsageError(command + " " + name + " appears more than once");
        }
        check_value(command, *f, words[i + 1]);
        o.text_[f->name] = words[i + 1];
    }
    for (const Flag& f : flags) {
        if (f.required && !o.given(f.name)) {
            throw UsageError(command + " needs " + f.name + " " + f.meta);
        }
        if (f.needs != nullptr && o.given(f.name) && !o.given(f.needs)) {
            throw UsageError(command + " " + f.name + " is only valid with " + f.needs);
        }
    }
    return o;
}

// --- JSON reports --------------------------------------------------------------------------

std::string json_text(const std::string& s)
{
    std::string out = "\"";
    for (const char c : s) {
        if (c == '"' || c == '\\') {
            out += '\\';
            out += c;
        } else if (static_cast<unsigned char>(c) < 0x20) {
            char esc[8];
            std::snprintf(esc, sizeof esc, "\\u%04x", static_cast<unsigned>(c));
            out += esc;
        } else {
            out += c;
        }
    }
    return out + "\"";
}

// Shortest decimal that reads back as the same double.
std::string json_number(double x)
{
    char buf[40];
    for (int digits = 15; digits <= 17; ++digits) {
        std::snprintf(buf, sizeof buf, "%.*g", digits, x);
        if (std::strtod(buf, nullptr) == x) {
            break;
        }
    }
    return buf;
}

class Json {
public:
    Json& put(const char* key, const std::string& v) { return raw(key, json_text(v)); }
    Json& put(const char* key, const char* v) { return raw(key, json_text(v)); }
    Json& put(const char* key, double v) { return raw(key, json_number(v)); }
    Json& put(const char* key, int v) { return raw(key, std::to_string(v)); }
    Json& put(const char* key, std::size_t v) { return raw(key, std::to_string(v)); }
    Json& put(const char* key, const PhaseTime& t)
    {
        return raw(key, Json().put("mean", t.mean_ms).put("std", t.std_ms).str());
    }
    Json& put(const char* key, const std::vector<std::string>& list)
    {
        std::vector<std::string> quoted;
        for (const std::string& s : list) {
            quoted.push_back(json_text(s));
        }
        return raw(key, "[" + joined(quoted, ", ") + "]");
    }
    Json& raw(const char* key, const std::string& value)
    {
        body_ += (body_.empty() ? "" : ", ") + json_text(key) + ": " + value;
        return *this;
    }
    std::string str() const { return "{" + body_ + "}"; }

private:
    std::string body_;
};

struct Device {
    cudaDeviceProp prop{};
    int runtime = 0;
    int driver = 0;

    static Device current()
    {
        Device d;
        int index = 0;
        CUDA_CHECK(cudaGetDevice(&index));
        CUDA_CHECK(cudaGetDeviceProperties(&d.prop, index));
        CUDA_CHECK(cudaRuntimeGetVersion(&d.runtime));
        CUDA_CHECK(cudaDriverGetVersion(&d.driver));
        return d;
    }
};

std::string cuda_version(int packed)  // 13000 -> "13.0"
{
    return std::to_string(packed / 1000) + "." + std::to_string(packed % 1000 / 10);
}

// What one compute subcommand did, for its report.
struct Done {
    const char* op;
    std::string impl;
    std::size_t num_in;
    std::size_t num_out;
};

// Without --bench, one line for a person; with it, the phase timings as one JSON object.
void report(const Options& o, const Done& d, const Bench& bench)
{
    if (!o.given("--bench")) {
        std::printf("rfgpu %s (%s): %zu input samples, %zu outputs written to %s\n", d.op,
                    d.impl.c_str(), d.num_in, d.num_out, o.text("--out").c_str());
        return;
    }
    const BenchResult& r = bench.result();
    Json j;
    j.put("op", d.op).put("impl", d.impl).put("gpu", Device::current().prop.name);
    j.put("num_in", d.num_in).put("num_out", d.num_out);
    j.put("runs", bench.config().runs).put("warmup", bench.config().warmup);
    j.put("h2d_ms", r.h2d).put("kernel_ms", r.kernel).put("d2h_ms", r.d2h);
    std::printf("%s\n", j.str().c_str());
}

// Rejects inputs whose element count does not fit the library's int lengths.
void fits_int(std::size_t n, const char* what)
{
    if (n > static_cast<std::size_t>(INT_MAX)) {
        throw std::runtime_error(std::string(what) + ": " + std::to_string(n) +
                                 " elements exceed the limit of " + std::to_string(INT_MAX));
    }
}

std::vector<float> taps_from(const Options& o)
{
    std::vector<float> taps = read_f32(o.text("--taps"));
    if (taps.empty()) {
        throw std::runtime_error(o.text("--taps") + ": the tap file holds no taps");
    }
    fits_int(taps.size(), "taps");
    return taps;
}

template <class Fn>
const Impl<Fn>& impl_named(const std::vector<Impl<Fn>>& table, const Options& o)
{
    const std::string name = o.text_or("--impl", table.front().name);
    for (const Impl<Fn>& row : table) {
        if (name == row.name) {
            return row;
        }
    }
    throw UsageError("no implementation named '" + name + "'");  // parse() checked it already
}

// --- the subcommands --------------------------------------------------------------------------

int do_fir(const Options& o)
{
    const Impl<FirFn>& impl = impl_named(fir_impls(), o);
    const int block = o.count_or("--block", kDefaultFirBlock);
    Bench bench(o.bench());
    StoredSamples x = read_stored(o.text("--in"));
    const std::vector<float> taps = taps_from(o);
    fits_int(x.count, "fir input");
    std::vector<cf32> y;
    if (x.count > 0 && x.format != SampleFormat::Cf32) {
        // Integer recordings are uploaded as stored and converted in the kernels' load stage.
        y = fir_stored(impl.name, x, taps, block, bench);
    } else if (x.count > 0) {
        const std::vector<cf32> samples = to_cf32(x);
        x.bytes.clear();
        x.bytes.shrink_to_fit();
        y = impl.fn(samples, taps, block, bench);
    }
    write_cf32(o.text("--out"), y);
    report(o, {"fir", impl.name, x.count, y.size()}, bench);
    return 0;
}

int do_channelize(const Options& o)
{
    const Impl<ChanFn>& impl = impl_named(channelize_impls(), o);
    const int channels = o.count_or("--channels", 1);
    const bool magnitude = o.text_or("--output", "complex") == "magnitude";
    Bench bench(o.bench());
    StoredSamples x = read_stored(o.text("--in"));
    const std::vector<float> taps = taps_from(o);
    fits_int(x.count + static_cast<std::size_t>(channels), "channelizer input with padding");
    std::vector<cf32> z;
    std::vector<float> mag;
    if (x.format != SampleFormat::Cf32) {
        channelize_stored(impl.name, x, taps, channels, magnitude, z, mag, bench);
    } else {
        const std::vector<cf32> samples = to_cf32(x);
        x.bytes.clear();
        x.bytes.shrink_to_fit();
        if (magnitude) {
            mag = channelize_magnitude(impl.name, samples, taps, channels, bench);
        } else {
            z = impl.fn(samples, taps, channels, bench);
        }
    }
    if (magnitude) {
        write_f32(o.text("--out"), mag);
    } else {
        write_cf32(o.text("--out"), z);
    }
    report(o, {"channelize", impl.name, x.count, magnitude ? mag.size() : z.size()}, bench);
    return 0;
}

// |x| of every sample (the project's magnitude subcommand, src/main.cpp:255-267).
int do_magnitude(const Options& o)
{
    Bench bench(o.bench());
    const std::vector<cf32> x = read_cf32(o.text("--in"));
    fits_int(x.size(), "magnitude input");
    const std::vector<float> mag = x.empty() ? std::vector<float>() : magnitude_cuda(x, bench);
    write_f32(o.text("--out"), mag);
    report(o, {"magnitude", "elementwise", x.size(), mag.size()}, bench);
    return 0;
}

// The streamed FIR. Without --bench: one pass written to --out. With --bench N: W untimed
// passes and N timed ones (wall clock of whole passes), reported with the throughput against
// --rate or the input's own sample rate.
int do_stream(const Options& o)
{
    StreamConfig config;
    const std::string impl = o.text_or("--impl", "tiled");
    parse_fir_impl(impl.c_str(), config.impl);  // parse() checked the name
    const std::string memory = o.text_or("--memory", "copy");
    parse_stream_memory(memory, config.memory);
    config.chunk = o.count_or("--chunk", config.chunk);
    config.depth = o.count_or("--depth", config.depth);
    const BenchConfig plan = o.bench();
    // Integer recordings stream as stored and are converted on the GPU.
    const StoredSamples x = read_stored(o.text("--in"));
    const std::vector<float> taps = taps_from(o);
    fits_int(x.count, "stream input");
    fits_int(static_cast<std::size_t>(config.chunk) + taps.size(), "chunk with its history");
    const double rate = o.given("--rate") ? o.real("--rate") : sample_rate(o.text("--in"));

    const bool timed = o.given("--bench");
    const int passes = timed ? plan.warmup + plan.runs : 1;
    std::vector<double> pass_ms;
    std::vector<cf32> y;
    StreamTiming timing;
    for (int i = 0; i < passes; ++i) {
        y = fir_stream(x, taps, config, timing);
        if (timed && i >= plan.warmup) {
            pass_ms.push_back(timing.total_ms);
        }
    }
    write_cf32(o.text("--out"), y);
    if (!timed) {
        std::printf("rfgpu stream (%s): %zu input samples in %d chunks of %d through %d slots, "
                    "written to %s\n",
                    impl.c_str(), x.count, timing.chunks, config.chunk, config.depth,
                    o.text("--out").c_str());
        return 0;
    }
    PhaseTime total;
    for (double t : pass_ms) {
        total.mean_ms += t / static_cast<double>(pass_ms.size());
    }
    if (pass_ms.size() > 1) {
        double ss = 0.0;
        for (double t : pass_ms) {
            ss += (t - total.mean_ms) * (t - total.mean_ms);
        }
        total.std_ms = std::sqrt(ss / static_cast<double>(pass_ms.size() - 1));
    }
    const double msps = total.mean_ms > 0 ? static_cast<double>(x.count) / total.mean_ms / 1e3
                                          : 0.0;
    Json j;
    j.put("op", "stream").put("impl", impl).put("memory", memory);
    j.put("gpu", Device::current().prop.name).put("num_in", x.count);
    j.put("chunk", config.chunk).put("depth", config.depth).put("chunks", timing.chunks);
    j.put("runs", plan.runs).put("warmup", plan.warmup).put("total_ms", total);
    j.put("msps", msps).put("sample_rate", rate);
    j.put("realtime_factor", rate > 0 ? msps * 1e6 / rate : 0.0);
    std::printf("%s\n", j.str().c_str());
    return 0;
}

int do_info(const Options&)
{
    const Device d = Device::current();
    const Json impls = Json()
                           .put("fir", fir_names())
                           .put("channelize", chan_names())
                           .put("magnitude", std::vector<std::string>{"elementwise"});
    Json j;
    j.put("gpu", d.prop.name);
    j.put("compute_capability",
          std::to_string(d.prop.major) + "." + std::to_string(d.prop.minor));
    j.put("memory_mb", static_cast<std::size_t>(d.prop.totalGlobalMem >> 20));
    j.put("sms", d.prop.multiProcessorCount);
    j.put("cuda_runtime", cuda_version(d.runtime)).put("cuda_driver", cuda_version(d.driver));
    j.put("library", rfx_version()).raw("impls", impls.str());
    std::printf("%s\n", j.str().c_str());
    return 0;
}

struct Command {
    const char* name;
    const char* purpose;
    std::vector<Flag> flags;
    int (*handler)(const Options&);
};

std::vector<Flag> with_bench(std::vector<Flag> flags)
{
    flags.push_back(count_flag("--bench", "N", 1));
    flags.push_back(count_flag("--warmup", "W", 0, INT_MAX, 1, false, "--bench"));
    return flags;
}

const std::vector<Command>& commands()
{
    static const std::vector<Command> table = {
        {"fir", "complex FIR filter, one output per input sample",
         with_bench({path_flag("--in", "X.cf32", true), path_flag("--taps", "H.f32", true),
                     path_flag("--out", "OUT.cf32", true),
                     word_flag("--impl", "NAME", fir_names),
                     count_flag("--block", "B", 32, 1024, 32)}),
         do_fir},
        {"channelize", "polyphase channelizer, frame-major channels (magnitude: |z| as float32)",
         with_bench({path_flag("--in", "X.cf32", true), path_flag("--taps", "H.f32", true),
                     count_flag("--channels", "M", 1, INT_MAX, 1, true),
                     path_flag("--out", "OUT", true), word_flag("--impl", "NAME", chan_names),
                     word_flag("--output", "complex|magnitude", output_names)}),
         do_channelize},
        {"magnitude", "|x| of every sample as float32",
         with_bench({path_flag("--in", "X.cf32", true), path_flag("--out", "OUT.f32", true)}),
         do_magnitude},
        {"stream", "FIR in chunks through a ring of D pinned buffers and CUDA streams",
         with_bench({path_flag("--in", "X.cf32", true), path_flag("--taps", "H.f32", true),
                     path_flag("--out", "OUT.cf32", true),
                     word_flag("--impl", "NAME", fir_names), count_flag("--chunk", "N", 1),
                     count_flag("--depth", "D", 1),
                     word_flag("--memory", "copy|registered|zero-copy", memory_names),
                     real_flag("--rate", "HZ")}),
         do_stream},
        {"info", "GPU, CUDA versions and implementations as JSON", {}, do_info},
    };
    return table;
}

template <class Fn>
void list_impls(const char* command, const std::vector<Impl<Fn>>& table)
{
    for (std::size_t i = 0; i < table.size(); ++i) {
        std::fprintf(stderr, "  %-11s --impl %-12s %s%s\n", command, table[i].name,
                     table[i].summary, i == 0 ? "  [default]" : "");
    }
}

void usage()
{
    std::fprintf(stderr, "usage: rfgpu COMMAND [--option value ...]\n\ncommands:\n");
    for (const Command& c : commands()) {
        std::string line = std::string("  rfgpu ") + c.name;
        for (const Flag& f : c.flags) {
            if (std::string(f.name) == "--bench" || std::string(f.name) == "--warmup") {
                continue;
            }
            const std::string item = std::string(f.name) + " " + f.meta;
            line += f.required ? " " + item : " [" + item + "]";
        }
        std::fprintf(stderr, "%s\n      %s\n", line.c_str(), c.purpose);
    }
    std::fprintf(stderr,
                 "\nSample inputs: .cf32 files or SigMF recordings (NAME.sigmf-meta or "
                 "NAME.sigmf-data)\nin cf32_le, ci16_le or ci8; integer recordings are "
                 "converted on the GPU.\n"
                 "Timing (fir, channelize, magnitude, stream): --bench N times N runs after "
                 "--warmup W\n(default 3) untimed ones and prints JSON.\n\nimplementations:\n");
    list_impls("fir", fir_impls());
    list_impls("channelize", channelize_impls());
}

}  // namespace

int main(int argc, char** argv)
{
    const std::string name = argc > 1 ? argv[1] : "";
    try {
        if (name == "--help" || name == "-h" || name == "help") {
            usage();
            return 0;
        }
        const auto& table = commands();
        const auto c = std::find_if(table.begin(), table.end(),
                                    [&](const Command& row) { return name == row.name; });
        if (c == table.end()) {
            throw UsageError(name.empty() ? "no command given"
                                          : "'" + name + "' is not a command");
        }
        const std::vector<std::string> words(argv + std::min(argc, 2), argv + argc);
        return c->handler(parse(c->name, c->flags, words));
    } catch (const UsageError& e) {
        std::fprintf(stderr, "rfgpu: %s\n\n", e.what());
        usage();
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "rfgpu: %s\n", e.what());
        return 1;
    }
}
