#pragma once

// Streaming FIR with the project's interface (src/stream.hpp:28-57): a capture processed in
// fixed-size chunks through a ring of `depth` slots, transfers of one chunk overlapping the
// kernel of another. The work is rfx_fir_stream (include/rfx.h); the result carries the same
// bits as filtering the whole capture at once with the same implementation.

#include "device_ops.hpp"
#include "io.hpp"
#include "types.hpp"

#include <string>
#include <vector>

enum class StreamMemory {
    Copy,        // host copies into and out of the pinned ring, async copies to the device
    Registered,  // input and output page-locked in place, async copies straight to and from them
    ZeroCopy,    // chunks move through mapped pinned memory, read and written by GPU kernels
};

struct StreamConfig {
    FirImpl impl = FirImpl::Tiled;
    int chunk = 1 << 20;  // samples per chunk
    int depth = 3;        // slots in the ring (and CUDA streams)
    StreamMemory memory = StreamMemory::Copy;
};

// "copy", "registered", or "zero-copy" (rfgpu stream --memory); false for anything else.
bool parse_stream_memory(const std::string& name, StreamMemory& memory);

struct StreamTiming {
    double total_ms = 0.0;  // wall clock from the first chunk to the last output on the host
    int chunks = 0;
};

// Output length x.size(). Allocation and the tap upload happen before the clock starts.
std::vector<cf32> fir_stream(const std::vector<cf32>& x, const std::vector<float>& taps,
                             const StreamConfig& config, StreamTiming& timing);

// The same over samples as stored (an integer SigMF recording): the stored bytes stream to the
// device and the kernels convert them (rfx_fir_stream_format); the bits of fir_stream over the
// converted samples.
std::vector<cf32> fir_stream(const StoredSamples& x, const std::vector<float>& taps,
                             const StreamConfig& config, StreamTiming& timing);
