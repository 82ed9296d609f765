#pragma once

// The operations as the command-line tool sees them, with the project's interface
// (src/ops.hpp:16-41): host data in, one-time setup outside the timed region, the upload /
// compute / download phases handed to Bench::run(), host data out.

#include "bench.hpp"
#include "io.hpp"
#include "types.hpp"

#include <vector>

template <class Fn>
struct Impl {
    const char* name;     // value of --impl
    const char* summary;  // one line for --help
    Fn fn;
};

// y[n] = sum_k taps[k] * x[n - k], x[m] = 0 for m < 0, output length x.size(). `block` is the
// project's --block (a multiple of 32 up to 1024); it does not change the result here.
using FirFn = std::vector<cf32> (*)(const std::vector<cf32>& x, const std::vector<float>& taps,
                                    int block, Bench& bench);
constexpr int kDefaultFirBlock = 256;
const std::vector<Impl<FirFn>>& fir_impls();  // first entry is the default

// The FIR of samples as stored (ci16 / ci8 SigMF recordings): the stored bytes are uploaded and
// converted in the kernels' load stage (rfx_fir_launch_format), with the results of converting
// on the host and running the implementation named `impl` (a fir_impls() name).
std::vector<cf32> fir_stored(const char* impl, const StoredSamples& x,
                             const std::vector<float>& taps, int block, Bench& bench);

// Polyphase channelizer: ceil(x.size() / channels) frames of `channels` values,
// z[t][k] = sum_l taps[l] * x[t*M - l] * exp(+2j*pi*k*l / M).
std::vector<cf32> channelize_cuda(const std::vector<cf32>& x, const std::vector<float>& taps,
                                  int channels, Bench& bench);

// mag[n] = |x[n]| (src/ops.hpp:27-29): one float per complex sample.
std::vector<float> magnitude_cuda(const std::vector<cf32>& x, Bench& bench);

// |channelize(x)| in one pass: frames x channels floats. `impl` is a channelize_impls() name;
// the tensor-core form takes the magnitude in its epilogue (rfx_channelize_magnitude_launch).
std::vector<float> channelize_magnitude(const char* impl, const std::vector<cf32>& x,
                                        const std::vector<float>& taps, int channels,
                                        Bench& bench);

// The channelizer of samples as stored (an integer SigMF recording), converted on the device:
// the results of channelizing the host-converted samples. `magnitude`: |z| per channel
// (frames x channels floats, returned as floats in `mag`), else z in `z`.
void channelize_stored(const char* impl, const StoredSamples& x, const std::vector<float>& taps,
                       int channels, bool magnitude, std::vector<cf32>& z, std::vector<float>& mag,
                       Bench& bench);

// The channelizer's implementations, selectable with --impl (the project has one).
using ChanFn = std::vector<cf32> (*)(const std::vector<cf32>& x, const std::vector<float>& taps,
                                     int channels, Bench& bench);
const std::vector<Impl<ChanFn>>& channelize_impls();  // first entry is the default
