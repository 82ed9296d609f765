// The project's streaming interface (src/stream.hpp) over rfx_fir_stream.
#include "stream.hpp"

#include "check.hpp"

#include <stdexcept>

bool parse_stream_memory(const std::string& name, StreamMemory& memory)
{
    if (name == "copy") {
        memory = StreamMemory::Copy;
    } else if (name == "registered") {
        memory = StreamMemory::Registered;
    } else if (name == "zero-copy") {
        memory = StreamMemory::ZeroCopy;
    } else {
        return false;
    }
    return true;
}

namespace {

std::vector<cf32> stream_samples(int format, const void* x, std::size_t count,
                                 const std::vector<float>& taps, const StreamConfig& config,
                                 StreamTiming& timing)
{
    if (config.chunk < 1 || config.depth < 1) {
        throw std::runtime_error("stream: chunk and depth must be at least 1");
    }
    std::vector<cf32> y(count);
    rfx_stream_config c{};
    c.impl = to_rfx_impl(config.impl);
    c.memory = config.memory == StreamMemory::Copy         ? RFX_STREAM_COPY
               : config.memory == StreamMemory::Registered ? RFX_STREAM_REGISTERED
                                                            : RFX_STREAM_ZERO_COPY;
    c.chunk = config.chunk;
    c.depth = config.depth;
    double total_ms = 0.0;
    int chunks = 0;
    RFX_CHECK(rfx_fir_stream_format(format, x, static_cast<int64_t>(count), taps.data(),
                                    static_cast<int>(taps.size()), &c, y.data(), &total_ms,
                                    &chunks));
    timing.total_ms = total_ms;
    timing.chunks = chunks;
    return y;
}

}  // namespace

std::vector<cf32> fir_stream(const std::vector<cf32>& x, const std::vector<float>& taps,
                             const StreamConfig& config, StreamTiming& timing)
{
    return stream_samples(RFX_FORMAT_CF32, x.data(), x.size(), taps, config, timing);
}

std::vector<cf32> fir_stream(const StoredSamples& x, const std::vector<float>& taps,
                             const StreamConfig& config, StreamTiming& timing)
{
    return stream_samples(static_cast<int>(x.format), x.bytes.data(), x.count, taps, config,
                          timing);
}
