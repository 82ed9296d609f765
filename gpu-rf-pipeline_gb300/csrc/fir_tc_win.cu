// Tensor-core FIR on sm_103a, resident-window form (2 to 385 taps): the block-Toeplitz GEMM
// of fir_tc.cu, tiled so that each sample crosses HBM and the copy engine once.
//
//   y[n] = sum_{k<K} h[k] x[n-k],  x[m < 0] = 0                              (src/fir.cu:1-5)
//
// Blocks of B = 128 outputs; a block reaches back C = floor((K + 126) / 128) blocks (1 to 3):
//   Y[:, j] = sum_{c=0}^{C} T_c X[:, j - c],   T_c(r, s) = h[cB + r - s]  (0 outside [0, K)).
// A tile is NB = 48 blocks (6144 outputs); its input window is blocks j0 - C .. j0 + 47. The
// GEMM per tile is D (128 x 96) += A (128 x 16) B (16 x 96) over K-steps (c, st): A is a
// descriptor into the tap strip (fir_tc.cu's layout: output rows stored reversed, so every 8 x 8
// core matrix of every T_c is one strip element), B the FP16 planes of K-step st (16 samples of
// each window row, N index 2 j + {0: I, 1: Q}). Chunk C of a K-step whose taps are all zero
// (16 st <= C B - K - 15) is skipped: 63 taps need 12 of the 16 chunk-steps.
//
// What differs from fir_tc.cu (which keeps the longer filters: at N = 96 the MMAs read 7 KB of
// operands per 48 tensor cycles, more than shared memory delivers, so from about 500 taps on
// fir_tc.cu's N = 192 tiles are faster: measured 123 against 120 us at 511 taps, 162 against
// 141 us at 1025):
//  * the whole window arrives by ONE 2-D TMA copy (rows of 1 KB for cf32) into a ring of three
//    window buffers, issued by a copy warp as soon as a buffer is converted: each sample
//    crosses HBM once and the TMA engine once (fir_tc.cu copies it twice: a scan slice and a
//    K-step box);
//  * the tile's power-of-two scale (largest |component| of the window brought into
//    [2^14, 2^15)) is a scan of that resident window by two scan warps as soon as it lands;
//    the eight producer warps only convert, from the same buffer, four K-steps at a time (a
//    thread's items of four K-steps are independent, so their loads, splits and stores overlap;
//    one K-step at a time took 62.7 us at 63 taps against 53.7 us);
//  * the large product h_hi x_hi goes to accumulator H in groups of whole K-steps of at most 18
//    MMAs (round-toward-zero accumulation: fir_tc.cu measured 5e-7 at 9 MMAs, 8e-7 at 18), H
//    double-buffered; the cross products go to X once per tile, X double-buffered: the MMAs of
//    one group or tile run while eight drain warps add the previous one into FP32 running sums.
// Split precision as in fir_tc.cu: x' = 2^ex x = x_hi + x_lo, h' = 2^eh h = h_hi + h_lo in FP16;
// the MMAs sum h_hi x_hi + h_hi x_lo + h_lo x_hi with FP32 accumulation; the drain scales by
// 2^-(ex + eh).
//
// The pipeline itself is in fir_tc_win.cuh (the batch kernel runs it over lists of captures).
//
// Roles (640 threads): warp 0 copies windows; warp 1 owns tensor memory and issues the MMAs (the
// warp runs the loop, one elected lane issues); warps 2-9 produce (FP16 hi/lo planes); warps
// 10-17 drain (warp w reads TMEM lane quarter w % 4, the columns of blocks 24 h .. 24 h + 23
// with h = (w - 10) / 4); warps 18-19 scan windows. Every wait is an mbarrier wait bounded in
// time, polled by every lane of a waiting warp (measured: lane 0 polling alone and handing the
// result to the warp by a shuffle took 18 us longer at 63 taps, the hand-off latency landing on
// every K-step); a give-up sets the fault word and every role stops.
#include "fir_tc.cuh"
#include "fir_tc_win.cuh"
#include "tmap.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_fir_tcw;

// wmap: x as rows of 256 components (one 128-sample block per row, full blocks only), boxes
// of 256 components x (48 + C) rows (one tile window). kFmt: 0 cf32, 1 ci16, 2 ci8 (the copy
// moves the components as stored; the producers decode them).
template <int C, int kFmt>
__global__ void __launch_bounds__(tcw::kThreads, 1)
fir_tcw_kernel(const __grid_constant__ CUtensorMap wmap, const void* __restrict__ x,
               const float* __restrict__ taps, float2* __restrict__ y, long long n, int num_taps,
               int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    tcw::Ctrl& ctl = *reinterpret_cast<tcw::Ctrl*>(smem);
    // The tensor-memory base travels through the last word of the control block's kilobyte.
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 1020);
    const int warp = threadIdx.x >> 5;
    if (warp == tcw::kMmaWarp) {
        tc::tmem_alloc(smem_u32(tmem_slot), tcw::kTmemCols);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot;
    const tcw::TcwSingleSrc src{&wmap, tcw::WinCapture{x, y, taps, n, num_taps, 0}, num_tiles};
    tcw::tcw_pipeline<C, kFmt, 8>(src, smem, ctl, tmem, &g_fault_fir_tcw);
    if (warp == tcw::kMmaWarp) {
        tc::tmem_dealloc(tmem, tcw::kTmemCols);
    }
}

bool fir_tcw_supported(int num_taps)
{
    return num_taps >= 2 && (num_taps + tcw::kB - 2) / tcw::kB <= tcw::kCMax &&
           tcw::win_layout((num_taps + tcw::kB - 2) / tcw::kB, 8, 1, 4).bytes <= tcw::kSmemMax;
}

long long fir_tcw_tile_outputs() { return static_cast<long long>(tcw::kNB) * tcw::kB; }

template <int C, int kFmt>
static cudaError_t launch_tcw(const void* x, const float* taps, void* y, long long n, int num_taps,
                              cudaStream_t stream)
{
    constexpr int es = tc::component_bytes(kFmt);
    const tcw::Layout lay = tcw::win_layout(C, 8, 1, es);
    if (lay.bytes > tcw::kSmemMax) {
        return cudaErrorInvalidValue;
    }
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) {
        return err;
    }
    int optin = 0;
    int sms = 0;
    if ((err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                      device)) != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    // At least 120 KB per block keeps one block per SM: each block owns all 512 TMEM columns.
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    if (bytes > static_cast<uint32_t>(optin)) {
        return cudaErrorInvalidValue;
    }
    err = cudaFuncSetAttribute(fir_tcw_kernel<C, kFmt>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    // x as rows of 256 components (one 128-sample block per row), full blocks only; one box
    // is a tile window.
    CUtensorMap map;
    err = encode_rows(&map, x, es, n / tcw::kB, 2 * tcw::kB, 2 * tcw::kB,
                      static_cast<uint32_t>(tcw::kNB + C));
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + tcw::kB - 1) / tcw::kB;
    const int tiles = static_cast<int>((blocks + tcw::kNB - 1) / tcw::kNB);
    const int grid = tiles < sms ? tiles : sms;
    fir_tcw_kernel<C, kFmt><<<grid, tcw::kThreads, bytes, stream>>>(
        map, x, taps, static_cast<float2*>(y), n, num_taps, tiles);
    return cudaGetLastError();
}

cudaError_t fir_tcw_launch(int format, const void* x, const float* taps, void* y, long long n,
                           int num_taps, cudaStream_t stream)
{
    if (n < tcw::kB || !fir_tcw_supported(num_taps)) {
        return cudaErrorInvalidValue;
    }
    const int C = (num_taps + tcw::kB - 2) / tcw::kB;
    if (format < 0 || format > 2) {
        return cudaErrorInvalidValue;
    }
    static cudaError_t (*const launchers[tcw::kCMax][3])(const void*, const float*, void*,
                                                          long long, int, cudaStream_t) = {
        {launch_tcw<1, 0>, launch_tcw<1, 1>, launch_tcw<1, 2>},
        {launch_tcw<2, 0>, launch_tcw<2, 1>, launch_tcw<2, 2>},
        {launch_tcw<3, 0>, launch_tcw<3, 1>, launch_tcw<3, 2>},
    };
    return launchers[C - 1][format](x, taps, y, n, num_taps, stream);
}

cudaError_t fir_tcw_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_tcw, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_tcw, &zero, sizeof(unsigned int));
}

}  // namespace rfx
