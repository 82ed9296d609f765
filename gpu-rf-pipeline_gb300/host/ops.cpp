// The project's operation interfaces (src/ops.hpp, src/device_ops.hpp) over the C ABI.
#include "device_buffer.hpp"
#include "device_ops.hpp"
#include "ops.hpp"

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

// ---- device-pointer entry points -----------------------------------------------------------

bool parse_fir_impl(const char* name, FirImpl& impl)
{
    static const struct {
        const char* name;
        FirImpl impl;
    } table[] = {{"naive", FirImpl::Naive},       {"tiled", FirImpl::Tiled},
                 {"tiled_const", FirImpl::TiledConst}, {"register", FirImpl::Register},
                 {"plain", FirImpl::Plain},       {"tc_split", FirImpl::TcSplit},
                 {"auto", FirImpl::Auto}};
    for (const auto& row : table) {
        if (std::strcmp(name, row.name) == 0) {
            impl = row.impl;
            return true;
        }
    }
    return false;
}

int to_rfx_impl(FirImpl impl)
{
    switch (impl) {
    case FirImpl::TcSplit: return RFX_FIR_TC;
    case FirImpl::Auto: return RFX_FIR_AUTO;
    default: return RFX_FIR_PLAIN;
    }
}

void fir_launch(FirImpl impl, const cf32* x, const float* taps, cf32* y, int num_samples,
                int num_taps, cudaStream_t stream)
{
    RFX_CHECK(rfx_fir_launch(to_rfx_impl(impl), x, taps, y, num_samples, num_taps, stream));
}

void fir_device(FirImpl impl, const cf32* x, const float* taps, cf32* y, int num_samples,
                int num_taps)
{
    RFX_CHECK(rfx_fir_device(to_rfx_impl(impl), x, taps, y, num_samples, num_taps));
}

void fir_load_const_taps(const float* taps, int num_taps, cudaStream_t stream)
{
    RFX_CHECK(rfx_fir_load_const_taps(taps, num_taps, stream));
}

void fir_naive_device(const cf32* x, const float* taps, cf32* y, int num_samples, int num_taps)
{
    fir_device(FirImpl::Naive, x, taps, y, num_samples, num_taps);
}

void fir_batched_device(FirImpl impl, const cf32* const* x, cf32* const* y,
                        const int* num_samples, int count, const float* taps, int num_taps)
{
    if (count < 1) {
        throw std::runtime_error("batched fir: " + std::to_string(count) +
                                 " channels, expected at least 1");
    }
    std::vector<const void*> xs(count);
    std::vector<void*> ys(count);
    std::vector<int64_t> ns(count);
    for (int c = 0; c < count; ++c) {
        xs[c] = x[c];
        ys[c] = y[c];
        ns[c] = num_samples[c];
    }
    RFX_CHECK(rfx_fir_batched_device(to_rfx_impl(impl), xs.data(), ys.data(), ns.data(), count,
                                     taps, num_taps, nullptr));
}

void fir_naive_batched_device(const cf32* const* x, cf32* const* y, const int* num_samples,
                              int count, const float* taps, int num_taps)
{
    fir_batched_device(FirImpl::Naive, x, y, num_samples, count, taps, num_taps);
}

int channelize_frames(int num_samples, int channels)
{
    return static_cast<int>(rfx_channelize_frames(num_samples, channels));
}

void channelize_device(cufftHandle plan, const cf32* x, const float* taps, cf32* out,
                       int num_samples, int channels, int num_taps)
{
    if (channelize_frames(num_samples, channels) == 0) {
        return;
    }
    RFX_CHECK(rfx_channelize_branches(x, taps, out, num_samples, channels, num_taps, nullptr));
    CUFFT_CHECK(cufftSetStream(plan, nullptr));
    CUFFT_CHECK(cufftExecC2C(plan, reinterpret_cast<cufftComplex*>(out),
                             reinterpret_cast<cufftComplex*>(out), CUFFT_INVERSE));
}

void channelize_device(rfx_chan_plan* plan, const cf32* x, const float* taps, cf32* out,
                       int num_samples, int num_taps, cudaStream_t stream)
{
    RFX_CHECK(rfx_channelize_launch(plan, x, taps, out, num_samples, num_taps, stream));
}

void channelize_magnitude_device(rfx_chan_plan* plan, const cf32* x, const float* taps,
                                 float* mag, int num_samples, int num_taps, cudaStream_t stream)
{
    RFX_CHECK(rfx_channelize_magnitude_launch(plan, x, taps, mag, num_samples, num_taps, stream));
}

void channelize_stored(const char* impl_name, const StoredSamples& x,
                       const std::vector<float>& taps, int channels, bool magnitude,
                       std::vector<cf32>& z, std::vector<float>& mag, Bench& bench)
{
    int impl = 0;
    RFX_CHECK(rfx_parse_chan_impl(impl_name, &impl));
    if (channels < 1) {
        throw std::runtime_error("channelize: need at least one channel");
    }
    const int num_samples = static_cast<int>(x.count);
    const int num_taps = static_cast<int>(taps.size());
    const int frames = channelize_frames(num_samples, channels);
    const std::size_t outputs = static_cast<std::size_t>(frames) * static_cast<std::size_t>(channels);
    z.assign(magnitude ? 0 : outputs, cf32{});
    mag.assign(magnitude ? outputs : 0, 0.0f);
    if (frames == 0) {
        return;
    }
    rfx_chan_plan* plan = nullptr;
    RFX_CHECK(rfx_chan_plan_create(impl, channels, num_samples, &plan));
    struct PlanGuard {
        rfx_chan_plan* p;
        ~PlanGuard() { rfx_chan_plan_destroy(p); }
    } guard{plan};
    DeviceBuffer<std::uint8_t> d_x(x.bytes.size());
    DeviceBuffer<float> d_h(taps.size());
    DeviceBuffer<cf32> d_out(outputs);   // |z| uses the first half of it
    bench.run(
        [&] {
            d_x.upload(x.bytes.data(), x.bytes.size());
            d_h.upload(taps.data(), taps.size());
        },
        [&] {
            RFX_CHECK(rfx_channelize_launch_format(
                plan, static_cast<int>(x.format),
                magnitude ? RFX_CHAN_OUT_MAGNITUDE : RFX_CHAN_OUT_COMPLEX, d_x.get(), d_h.get(),
                d_out.get(), num_samples, num_taps, nullptr));
        },
        [&] {
            if (magnitude) {
                CUDA_CHECK(cudaMemcpy(mag.data(), d_out.get(), outputs * sizeof(float),
                                      cudaMemcpyDeviceToHost));
            } else {
                d_out.download(z.data(), outputs);
            }
        });
}

void magnitude_device(const cf32* x, float* mag, int num_samples)
{
    RFX_CHECK(rfx_magnitude_launch(x, mag, num_samples, nullptr));
}

std::vector<float> magnitude_cuda(const std::vector<cf32>& x, Bench& bench)
{
    const int num_samples = static_cast<int>(x.size());
    std::vector<float> mag(x.size());
    DeviceBuffer<cf32> d_x(x.size());
    DeviceBuffer<float> d_mag(mag.size());
    bench.run([&] { d_x.upload(x.data(), x.size()); },
              [&] { magnitude_device(d_x.get(), d_mag.get(), num_samples); },
              [&] { d_mag.download(mag.data(), mag.size()); });
    return mag;
}

std::vector<float> channelize_magnitude(const char* impl_name, const std::vector<cf32>& x,
                                        const std::vector<float>& taps, int channels,
                                        Bench& bench)
{
    int impl = 0;
    RFX_CHECK(rfx_parse_chan_impl(impl_name, &impl));
    if (channels < 1) {
        throw std::runtime_error("channelize: need at least one channel");
    }
    const int num_samples = static_cast<int>(x.size());
    const int num_taps = static_cast<int>(taps.size());
    const int frames = channelize_frames(num_samples, channels);
    std::vector<float> mag(static_cast<std::size_t>(frames) * static_cast<std::size_t>(channels));
    if (frames == 0) {
        return mag;
    }
    rfx_chan_plan* plan = nullptr;
    RFX_CHECK(rfx_chan_plan_create(impl, channels, num_samples, &plan));
    struct PlanGuard {
        rfx_chan_plan* p;
        ~PlanGuard() { rfx_chan_plan_destroy(p); }
    } guard{plan};
    DeviceBuffer<cf32> d_x(x.size());
    DeviceBuffer<float> d_h(taps.size());
    DeviceBuffer<float> d_mag(mag.size());
    bench.run(
        [&] {
            d_x.upload(x.data(), x.size());
            d_h.upload(taps.data(), taps.size());
        },
        [&] {
            channelize_magnitude_device(plan, d_x.get(), d_h.get(), d_mag.get(), num_samples,
                                        num_taps);
        },
        [&] { d_mag.download(mag.data(), mag.size()); });
    return mag;
}

// ---- host-vector operations ----------------------------------------------------------------

namespace {

std::vector<cf32> fir_host(FirImpl impl, const std::vector<cf32>& x,
                           const std::vector<float>& taps, int block, Bench& bench)
{
    if (block < 32 || block > 1024 || block % 32 != 0) {
        throw std::runtime_error("fir: block " + std::to_string(block) +
                                 " is not a multiple of 32 up to 1024");
    }
    const int num_samples = static_cast<int>(x.size());
    const int num_taps = static_cast<int>(taps.size());
    std::vector<cf32> y(x.size());
    RFX_CHECK(rfx_fir_load_const_taps(taps.data(), num_taps, nullptr));  // capacity check only
    DeviceBuffer<cf32> d_x(x.size());
    DeviceBuffer<cf32> d_y(y.size());
    DeviceBuffer<float> d_h(taps.size());
    bench.run(
        [&] {
            d_x.upload(x.data(), x.size());
            d_h.upload(taps.data(), taps.size());
        },
        [&] { fir_launch(impl, d_x.get(), d_h.get(), d_y.get(), num_samples, num_taps, nullptr); },
        [&] { d_y.download(y.data(), y.size()); });
    return y;
}

#define RFX_FIR_ENTRY(fn, impl)                                                                  \
    std::vector<cf32> fn(const std::vector<cf32>& x, const std::vector<float>& taps, int block,  \
                         Bench& bench)                                                           \
    {                                                                                            \
        return fir_host(impl, x, taps, block, bench);                                            \
    }

RFX_FIR_ENTRY(fir_plain, FirImpl::Plain)
RFX_FIR_ENTRY(fir_tc_split, FirImpl::TcSplit)
RFX_FIR_ENTRY(fir_auto, FirImpl::Auto)
RFX_FIR_ENTRY(fir_naive, FirImpl::Naive)
RFX_FIR_ENTRY(fir_tiled, FirImpl::Tiled)
RFX_FIR_ENTRY(fir_tiled_const, FirImpl::TiledConst)
RFX_FIR_ENTRY(fir_register, FirImpl::Register)

}  // namespace

std::vector<cf32> fir_stored(const char* impl_name, const StoredSamples& x,
                             const std::vector<float>& taps, int block, Bench& bench)
{
    if (block < 32 || block > 1024 || block % 32 != 0) {
        throw std::runtime_error("fir: block " + std::to_string(block) +
                                 " is not a multiple of 32 up to 1024");
    }
    FirImpl impl;
    if (!parse_fir_impl(impl_name, impl)) {
        throw std::runtime_error(std::string("fir: unknown implementation ") + impl_name);
    }
    const int num_samples = static_cast<int>(x.count);
    const int num_taps = static_cast<int>(taps.size());
    std::vector<cf32> y(x.count);
    RFX_CHECK(rfx_fir_load_const_taps(taps.data(), num_taps, nullptr));  // capacity check only
    DeviceBuffer<std::uint8_t> d_x(x.bytes.size());
    DeviceBuffer<cf32> d_y(y.size());
    DeviceBuffer<float> d_h(taps.size());
    bench.run(
        [&] {
            d_x.upload(x.bytes.data(), x.bytes.size());
            d_h.upload(taps.data(), taps.size());
        },
        [&] {
            RFX_CHECK(rfx_fir_launch_format(to_rfx_impl(impl), static_cast<int>(x.format),
                                            d_x.get(), d_h.get(), d_y.get(), num_samples,
                                            num_taps, nullptr));
        },
        [&] { d_y.download(y.data(), y.size()); });
    return y;
}

namespace {

std::vector<cf32> channelize_impl(int impl, const std::vector<cf32>& x,
                                  const std::vector<float>& taps, int channels, Bench& bench)
{
    if (channels < 1) {
        throw std::runtime_error("channelize: need at least one channel");
    }
    const int num_samples = static_cast<int>(x.size());
    const int num_taps = static_cast<int>(taps.size());
    const int frames = channelize_frames(num_samples, channels);
    std::vector<cf32> z(static_cast<std::size_t>(frames) * static_cast<std::size_t>(channels));
    if (frames == 0) {
        return z;
    }
    // One-time setup outside the timed region: buffers and the plan (cuFFT plan or twiddles).
    rfx_chan_plan* plan = nullptr;
    RFX_CHECK(rfx_chan_plan_create(impl, channels, num_samples, &plan));
    struct PlanGuard {
        rfx_chan_plan* p;
        ~PlanGuard() { rfx_chan_plan_destroy(p); }
    } guard{plan};
    DeviceBuffer<cf32> d_x(x.size());
    DeviceBuffer<float> d_h(taps.size());
    DeviceBuffer<cf32> d_z(z.size());
    bench.run(
        [&] {
            d_x.upload(x.data(), x.size());
            d_h.upload(taps.data(), taps.size());
        },
        [&] { channelize_device(plan, d_x.get(), d_h.get(), d_z.get(), num_samples, num_taps); },
        [&] { d_z.download(z.data(), z.size()); });
    return z;
}

std::vector<cf32> channelize_plain(const std::vector<cf32>& x, const std::vector<float>& taps,
                                   int channels, Bench& bench)
{
    return channelize_impl(RFX_CHAN_PLAIN, x, taps, channels, bench);
}

std::vector<cf32> channelize_tc(const std::vector<cf32>& x, const std::vector<float>& taps,
                                int channels, Bench& bench)
{
    return channelize_impl(RFX_CHAN_TC, x, taps, channels, bench);
}

std::vector<cf32> channelize_auto(const std::vector<cf32>& x, const std::vector<float>& taps,
                                  int channels, Bench& bench)
{
    return channelize_impl(RFX_CHAN_AUTO, x, taps, channels, bench);
}

}  // namespace

const std::vector<Impl<FirFn>>& fir_impls()
{
    static const std::vector<Impl<FirFn>> impls = {
        {"plain", "FP32 CUDA cores: TMA-staged tile, 9 outputs/thread, f32x2 FMA", fir_plain},
        {"tc_split", "tcgen05 block-Toeplitz GEMM, split FP16, FP32 accumulate", fir_tc_split},
        {"auto", "the tuned choice for this tap count and length", fir_auto},
        {"naive", "the project's name; runs plain (same results bit for bit)", fir_naive},
        {"tiled", "the project's name; runs plain (same results bit for bit)", fir_tiled},
        {"tiled_const", "the project's name; runs plain (same results bit for bit)",
         fir_tiled_const},
        {"register", "the project's name; runs plain (same results bit for bit)", fir_register},
    };
    return impls;
}

const std::vector<Impl<ChanFn>>& channelize_impls()
{
    static const std::vector<Impl<ChanFn>> impls = {
        {"plain", "FP32 branch sums + cuFFT batched inverse FFT", channelize_plain},
        {"tc_split", "DFT as a split-FP16 tcgen05 GEMM: fused with the FP32 branch sums (64 ch); "
                     "32 x 32 factored after them (1024 ch)",
         channelize_tc},
        {"auto", "tc_split for 64 channels, plain otherwise", channelize_auto},
    };
    return impls;
}

std::vector<cf32> channelize_cuda(const std::vector<cf32>& x, const std::vector<float>& taps,
                                  int channels, Bench& bench)
{
    return channelize_plain(x, taps, channels, bench);
}
