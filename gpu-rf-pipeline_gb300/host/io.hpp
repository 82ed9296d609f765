#pragma once

// Raw little-endian sample files (src/io.hpp): .cf32 = interleaved float32 I/Q, .f32 = float32
// taps. Errors throw std::runtime_error naming the file.

#include "types.hpp"

#include <string>
#include <vector>

std::vector<cf32> read_cf32(const std::string& path);
std::vector<float> read_f32(const std::string& path);
void write_cf32(const std::string& path, const std::vector<cf32>& x);
void write_f32(const std::string& path, const std::vector<float>& x);

// Sample rate in Hz from the PATH.json sidecar the project's fixture generator writes next to
// a .cf32 file ("sample_rate" field); 0 when there is none (src/io.hpp:27-30).
double sample_rate(const std::string& path);
