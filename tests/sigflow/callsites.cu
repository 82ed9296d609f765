// Test program shaped like the CUDA code the project's SigFlow compiler generates
// (compiler/src/backend_cuda.cpp): the same includes, a `sigflow::Runtime rt`, buffer slots,
// taps and cuFFT plans from the runtime, and inside rt.run the generated call forms —
//   fused FIR group:  fir_batched_device(FirImpl::K, x, y, n, count, t, taps)      (:306-340)
//                     fir_naive_batched_device(x, y, n, count, t, taps)            (fir=naive)
//   single FIR:       fir_device(FirImpl::K, in, t, out, static_cast<int>(n), taps) (:224-236)
//                     fir_naive_device(in, t, out, static_cast<int>(n), taps)      (fir=naive)
//   channelizer:      channelize_device(plan, in, t, out, static_cast<int>(n), M, taps)
//                                                                                   (:272-277)
//   magnitude:        magnitude_device(in, out, static_cast<int>(n))
// compiled against this library's device_ops.hpp and linked with librfxhost.a + librfx.so.
// Build with -DSIGFLOW_FIR_NAIVE=1 for the fir=naive forms. Run from a directory holding
// fixtures/ (tone.cf32, tone_odd.cf32, lowpass.f32, lowpass_long.f32, channelizer_proto.f32)
// and an out/ directory.
#include "device_ops.hpp"
#include "pipeline_runtime.hpp"

#include <cstdio>
#include <exception>
#include <vector>

int main(int argc, char** argv)
try {
#if SIGFLOW_FIR_NAIVE
    sigflow::Runtime rt("callsites.sf", "fir=naive xcorr=naive", true, true, argc, argv);
#else
    sigflow::Runtime rt("callsites.sf", "fir=tiled_const xcorr=naive", true, true, argc, argv);
#endif

    // Captures, read once.
    const std::vector<cf32> h0 = rt.read_capture("fixtures/tone.cf32");
    const std::vector<cf32> h1 = rt.read_capture("fixtures/tone_odd.cf32");

    // Samples in every value.
    const std::size_t n0 = h0.size();
    const std::size_t n1 = h1.size();
    const std::size_t n2 = n0;                                   // fir %0 lowpass [fused 0]
    const std::size_t n3 = n1;                                   // fir %1 lowpass [fused 0]
    const std::size_t n4 = n0;                                   // fir %0 lowpass_long
    const std::size_t n5 = sigflow::padded_to_frames(n0, 16);    // channelize %0, 16 channels
    const std::size_t n6 = n5;                                   // magnitude %5
    const std::size_t n7 = sigflow::padded_to_frames(n1, 64);    // channelize %1, 64 channels

    // Buffer slots.
    rt.need(0, n0 * sizeof(cf32));
    rt.need(1, n1 * sizeof(cf32));
    rt.need(2, n2 * sizeof(cf32));
    rt.need(3, n3 * sizeof(cf32));
    rt.need(4, n4 * sizeof(cf32));
    rt.need(5, n5 * sizeof(cf32));
    rt.need(6, n6 * sizeof(float));
    rt.need(7, n7 * sizeof(cf32));
    rt.allocate_slots();

    // Taps and FFT plans.
    int taps2 = 0;
    const float* t2 = rt.taps("fixtures/lowpass.f32", taps2);
    int taps4 = 0;
    const float* t4 = rt.taps("fixtures/lowpass_long.f32", taps4);
    int taps5 = 0;
    const float* t5 = rt.taps("fixtures/channelizer_proto.f32", taps5);
    const cufftHandle plan5 = rt.fft_plan(16, n5 / 16);
    int taps7 = 0;
    const float* t7 = rt.taps("fixtures/lowpass_long.f32", taps7);
    const cufftHandle plan7 = rt.fft_plan(64, n7 / 64);

    // Host copies of the emitted values.
    std::vector<cf32> out8(n2);
    std::vector<cf32> out9(n3);
    std::vector<cf32> out10(n4);
    std::vector<cf32> out11(n5);
    std::vector<float> out12(n6);
    std::vector<cf32> out13(n7);

    rt.run(
        [&] {
            CUDA_CHECK(cudaMemcpy(rt.slot<cf32>(0), h0.data(), n0 * sizeof(cf32), cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(rt.slot<cf32>(1), h1.data(), n1 * sizeof(cf32), cudaMemcpyHostToDevice));
        },
        [&] {
            {  // fusion group 0: 2 FIRs, one launch
                const cf32* x[] = {rt.slot<cf32>(0), rt.slot<cf32>(1)};
                cf32* y[] = {rt.slot<cf32>(2), rt.slot<cf32>(3)};
                const int n[] = {static_cast<int>(n2), static_cast<int>(n3)};
#if SIGFLOW_FIR_NAIVE
                fir_naive_batched_device(x, y, n, 2, t2, taps2);
#else
                fir_batched_device(FirImpl::TiledConst, x, y, n, 2, t2, taps2);
#endif
                rt.count("fir_batched");
            }
#if SIGFLOW_FIR_NAIVE
            fir_naive_device(rt.slot<cf32>(0), t4, rt.slot<cf32>(4), static_cast<int>(n4), taps4);
#else
            fir_device(FirImpl::TiledConst, rt.slot<cf32>(0), t4, rt.slot<cf32>(4), static_cast<int>(n4), taps4);
#endif
            rt.count("fir");
            channelize_device(plan5, rt.slot<cf32>(0), t5, rt.slot<cf32>(5), static_cast<int>(n0), 16, taps5);
            rt.count("channelize");
            rt.count("cufft");
            magnitude_device(rt.slot<cf32>(5), rt.slot<float>(6), static_cast<int>(n6));
            rt.count("magnitude");
            channelize_device(plan7, rt.slot<cf32>(1), t7, rt.slot<cf32>(7), static_cast<int>(n1), 64, taps7);
            rt.count("channelize");
            rt.count("cufft");
        },
        [&] {
            CUDA_CHECK(cudaMemcpy(out8.data(), rt.slot<cf32>(2), n2 * sizeof(cf32), cudaMemcpyDeviceToHost));
            CUDA_CHECK(cudaMemcpy(out9.data(), rt.slot<cf32>(3), n3 * sizeof(cf32), cudaMemcpyDeviceToHost));
            CUDA_CHECK(cudaMemcpy(out10.data(), rt.slot<cf32>(4), n4 * sizeof(cf32), cudaMemcpyDeviceToHost));
            CUDA_CHECK(cudaMemcpy(out11.data(), rt.slot<cf32>(5), n5 * sizeof(cf32), cudaMemcpyDeviceToHost));
            CUDA_CHECK(cudaMemcpy(out12.data(), rt.slot<float>(6), n6 * sizeof(float), cudaMemcpyDeviceToHost));
            CUDA_CHECK(cudaMemcpy(out13.data(), rt.slot<cf32>(7), n7 * sizeof(cf32), cudaMemcpyDeviceToHost));
        });

    rt.write_cf32("out/fir_a.cf32", out8);
    rt.write_cf32("out/fir_b.cf32", out9);
    rt.write_cf32("out/fir_long.cf32", out10);
    rt.write_cf32("out/ch16.cf32", out11);
    rt.write_f32("out/ch16_mag.f32", out12);
    rt.write_cf32("out/ch64.cf32", out13);
    rt.report();
    return 0;
} catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
}
