#pragma once

// Raw little-endian sample files (src/io.hpp): .cf32 = interleaved float32 I/Q, .f32 = float32
// taps. Every sample input may also be a SigMF recording, named by either file of the pair
// (NAME.sigmf-meta, NAME.sigmf-data; src/io.hpp:21-25): cf32_le, ci16_le or ci8/ci8_le, one
// channel. Errors throw std::runtime_error naming the file.

#include "types.hpp"

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

bool is_sigmf(const std::string& path);

// The stored form of a sample input: .cf32 files are Cf32; a SigMF recording has its
// core:datatype. Values match rfx_sample_format.
enum class SampleFormat { Cf32 = 0, Ci16 = 1, Ci8 = 2 };
SampleFormat sample_format(const std::string& path);

// The input's samples as stored (count samples of 8, 4 or 2 bytes), for conversion on the
// device (rfx_fir_launch_format).
struct StoredSamples {
    SampleFormat format = SampleFormat::Cf32;
    std::size_t count = 0;
    std::vector<std::uint8_t> bytes;
};
StoredSamples read_stored(const std::string& path);

// cf32 samples: a .cf32 file as is, a SigMF recording converted as the project converts it
// (src/io.cpp:110-148): ci16 components v / 32768, ci8 components v / 128.
std::vector<cf32> read_cf32(const std::string& path);
std::vector<cf32> to_cf32(const StoredSamples& stored);
std::vector<float> read_f32(const std::string& path);
void write_cf32(const std::string& path, const std::vector<cf32>& x);
void write_f32(const std::string& path, const std::vector<float>& x);

// Sample rate in Hz: core:sample_rate of a SigMF recording, else the "sample_rate" field of the
// PATH.json sidecar the project's fixture generator writes next to a .cf32 file; 0 when there
// is none (src/io.hpp:27-30, src/io.cpp:157-173).
double sample_rate(const std::string& path);
