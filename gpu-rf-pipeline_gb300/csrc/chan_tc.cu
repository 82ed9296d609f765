// Tensor-core polyphase channelizer for sm_103a, M = 64 channels, one fused kernel.
//
//   u[t][m] = sum_p h[pM + m] x[tM - pM - m]            (x[i < 0] = 0)      src/channelize.cu:25-49
//   z[t][k] = sum_m u[t][m] e^{+2 pi i k m / M}                              src/channelize.cu:70-71
//
// Per tile of 128 frames (8192 samples):
//  1. Samples arrive by 2-D TMA copies (rows = frames of 64 samples, zero fill outside the
//     input) in two half-windows: frames [t0 + 64 h, +64) need rows t0 + 64 h - P .. +63
//     (P = taps per branch), i.e. 64 + P rows per half, double-buffered so the next tile's
//     samples stream in while this tile is finished.
//  2. Branch sums on CUDA cores, FP32, from shared memory: warps 0-7 read half-window 0,
//     warps 8-15 half-window 1; lane l owns branches (64 - l) % 64 and 32 - l (window columns
//     l and 32 + l, so a warp's loads are conflict-free) for 8 consecutive frames. For one
//     branch the frames form a FIR over the decimated sequence s_d = x[(t0 + d) M - m] with
//     taps g_p = h[pM + m] (from shared memory up to 26 taps per branch, else the L1 cache);
//     two alternating 8-sample register blocks, taps in ascending p, one packed f32x2 fused
//     multiply-add per tap: each sample loaded serves eight frames.
//  3. Each frame's largest |u| sets a power-of-two scale for that frame (one GEMM row; the
//     drain undoes it row by row); u' = u_hi + u_lo in FP16 is written as
//     the GEMM's A operand (rows = frames, K = [Re u, Im u] in the lanes' branch order:
//     K index 2l -> branch (64 - l) % 64, 2l + 1 -> 32 - l; W's rows follow the same order).
//  4. The DFT as a real GEMM: [Re z, Im z] (128 x 128) = A (128 x 128) W, with
//     W = [[cos, sin], [-sin, cos]](2 pi k m / M) built in FP64 on the GPU (rfx_chan_plan_create)
//     and split hi/lo once; three split products per K-step on tcgen05 (M=128, N=128, K=16).
//     The tensor core accumulates FP32 with round-toward-zero, so two TMEM accumulators take
//     twelve MMAs each and are summed in FP32 registers; the accumulators are double-buffered
//     (2 tiles x 2 x 128 columns) so the MMAs of tile k + 1 run while tile k is drained.
//  5. Scale back by 2^-(eu + ew) and store each frame's 64 channels. The accumulator columns
//     are ordered (column_to_channel) so that 16x256b tensor-memory loads hand four adjacent
//     lanes a frame's channels in pairs: each store instruction writes 64 contiguous bytes of
//     eight frames (whole 32-byte sectors) instead of 16 bytes of 32 frames.
//
// Roles (576 threads): warps 0-15 compute branch sums, write operands and drain the
// accumulators (warp w: TMEM lane quarter w % 4 = frames 32 (w % 4) .. +31, accumulator
// columns 32 (w / 4) .. +31 = channels 16 (w / 4) .. +15); warp 16 owns tensor memory and
// issues the MMAs; warp 17 refills the half-windows as their eight warps release them. The loop runs the branch
// sums of tile k + 1 and stages its operand before draining tile k, so the MMAs of tile k hide
// behind the branch sums and those of tile k + 1 behind the drain. Every wait is a bounded
// mbarrier wait.
#include "chan_tc.cuh"
#include "magnitude.cuh"
#include "tc_common.cuh"
#include "tmap.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_chan_tc;

namespace {

using namespace tc;

constexpr int kM = 64;                 // channels
constexpr int kK = 2 * kM;             // GEMM K and N: Re and Im parts
constexpr int kFrames = 128;           // frames per tile = MMA M
constexpr int kHalf = kFrames / 2;     // frames per half-window
constexpr int kWorkerWarpsConst = 16;
constexpr int kR = 8;                  // frames per thread (one half-window per warp)
constexpr int kHalfWarps = kWorkerWarpsConst / 2;  // worker warps per half-window
constexpr int kWorkerWarps = kWorkerWarpsConst;
constexpr int kMmaWarp = 16;
constexpr int kTmaWarp = 17;
constexpr int kThreads = 18 * 32;
constexpr int kParts = 2;              // TMEM accumulators per tile, 4 K-steps each
constexpr uint32_t kTmemCols = 512;    // 2 tiles x kParts x kK
constexpr uint32_t kPlane = kFrames * 16 + 16;  // bytes per 8-element K plane (+16: banks)
constexpr uint32_t kSplit = (kK / 8) * kPlane;  // one split of one operand
constexpr uint32_t kIdesc = idesc_f16(kFrames, kK);
constexpr int kWExp = 14;              // W' = 2^14 W, |W| <= 1
constexpr int kMaxPerBranch = 32;      // taps per branch the kernel takes
constexpr int kSmemTapsMax = 26;       // taps per branch up to which the taps sit in smem too
constexpr int kColsPerSlice = 32;      // accumulator columns a drain warp reads: 16 channels
// Tiles whose frame exponents are kept: tile k's are rewritten at tile k + kExpBufs, by which
// time every worker has drained tile k (staging tile k + 4 needs the MMAs of tile k + 3, which
// need every worker's operand of tile k + 3, staged after its drain of tile k + 1).
constexpr int kExpBufs = 4;

// The GEMM's N index (accumulator column) -> output channel and part (0 Re, 1 Im). Column
// 32 s + 8 j + 2 q + b holds part b of channel 16 s + 8 (j / 2) + 2 q + j % 2, so that the
// drain's 16x256b loads give thread q of a frame (Re, Im) of channels c and c + 1 side by
// side (c = 16 s + 8 (j / 2) + 2 q): one 16-byte store.
__host__ __device__ inline void column_to_channel(int n, int& ch, int& part)
{
    const int s = n >> 5;
    const int j = (n >> 3) & 3;
    const int q = (n >> 1) & 3;
    part = n & 1;
    ch = 16 * s + 8 * (j >> 1) + 2 * q + (j & 1);
}

// The GEMM's K index of Re u (k < 64; Im u at 64 + k) -> branch. Lane l owns K indices 2l and
// 2l + 1, i.e. branches (64 - l) % 64 and 32 - l, whose window columns (64 - m) % 64 are l and
// 32 + l: a warp's window loads read 32 consecutive 8-byte columns (no bank conflicts).
__host__ __device__ inline int k_to_branch(int k)
{
    const int l = k >> 1;
    return (k & 1) ? 32 - l : (64 - l) & 63;
}

struct Layout {
    int P;                 // taps per branch
    int wrows;             // rows per half-window: kHalf + P
    uint32_t win;          // bytes per half-window
    uint32_t w_hi, w_lo, a_hi, a_lo, win0, taps, bytes;
};

// sb: bytes per input sample as stored (8 cf32, 4 ci16, 2 ci8).
__host__ __device__ inline Layout chan_layout(int num_taps, int sb = 8)
{
    Layout l;
    l.P = (num_taps + kM - 1) / kM;
    l.wrows = kHalf + l.P;
    l.win = static_cast<uint32_t>(l.wrows) * kM * static_cast<uint32_t>(sb);
    l.w_hi = 1024;
    l.w_lo = l.w_hi + kSplit;
    l.a_hi = l.w_lo + kSplit;
    l.a_lo = l.a_hi + kSplit;
    l.win0 = l.a_lo + kSplit;                     // two half-window buffers
    l.taps = l.win0 + 2u * l.win;                 // taps[p][slot], slot = the lane's column
    l.bytes = l.taps + (l.P <= kSmemTapsMax ? static_cast<uint32_t>(l.P) * kM * 4u : 0u);
    return l;
}

struct Ctrl {
    unsigned long long full;
    unsigned long long empty;
    unsigned long long win_full[2];
    unsigned long long win_empty[2];
    unsigned long long dfull[2];
    unsigned long long dempty[2];
    unsigned long long eready[kExpBufs];  // the frame exponents of a tile are written
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    signed char fexp[kExpBufs][kFrames];  // frame scale exponents (clamped to 127)
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// Taps p0 + q (q < nq) of one branch: acc[i] += g_p s_{i - p} with cur = S_g, nxt = S_{g+1},
// S_g[i] = s_{-8g + i}. The taps come from shared memory (tap_s: the branch's column of the
// taps[p][slot] table, 256 bytes per p) or, for the longest filters, through the L1 cache.
template <bool kTapsSmem>
__device__ __forceinline__ void branch_group(f32x2 (&acc)[kR], const f32x2 (&cur)[kR],
                                             const f32x2 (&nxt)[kR], const float* __restrict__ taps,
                                             uint32_t tap_s, int m, int p0, int nq, int num_taps)
{
#pragma unroll
    for (int q = 0; q < kR; ++q) {
        if (q < nq) {
            float hv;
            if (kTapsSmem) {
                asm volatile("ld.shared.f32 %0, [%1];"
                             : "=f"(hv)
                             : "r"(tap_s + static_cast<uint32_t>(p0 + q) * (kM * 4u)));
            } else {
                const int l = (p0 + q) * kM + m;
                hv = l < num_taps ? __ldg(taps + l) : 0.0f;
            }
            const f32x2 h2 = pack2(hv, hv);
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                acc[i] = fma2(h2, i >= q ? cur[i - q] : nxt[kR + i - q], acc[i]);
            }
        }
    }
}

// Sample formats of x (rfx_sample_format): 0 cf32; 1 ci16 and 2 ci8, whose components are
// converted as the project's SigMF reader converts them (src/io.cpp:110-148: v / 32768, v / 128,
// exact in float32) where the window is read, so the results are those of the converted input.
__host__ __device__ constexpr int sample_bytes(int fmt) { return fmt == 0 ? 8 : fmt == 1 ? 4 : 2; }

template <int kFmt>
__device__ __forceinline__ f32x2 lds_sample(uint32_t addr)
{
    if constexpr (kFmt == 0) {
        return lds64(addr);
    } else if constexpr (kFmt == 1) {
        uint32_t w;
        asm volatile("ld.shared.u32 %0, [%1];" : "=r"(w) : "r"(addr));
        return pack2(static_cast<float>(static_cast<int>(w << 16) >> 16) * (1.0f / 32768.0f),
                     static_cast<float>(static_cast<int>(w) >> 16) * (1.0f / 32768.0f));
    } else {
        unsigned short w;
        asm volatile("ld.shared.u16 %0, [%1];" : "=h"(w) : "r"(addr));
        const int v = w;
        return pack2(static_cast<float>(static_cast<int>(static_cast<uint32_t>(v) << 24) >> 24) *
                         (1.0f / 128.0f),
                     static_cast<float>(static_cast<int>(static_cast<uint32_t>(v) << 16) >> 24) *
                         (1.0f / 128.0f));
    }
}

}  // namespace

// kMag: the output is |z| (float per channel, frames x 64) instead of z (cf32), computed from
// the same floats z would hold.
template <bool kTapsSmem, bool kMag, int kFmt>
__global__ void __launch_bounds__(kThreads, 1)
chan_tc_kernel(const __grid_constant__ CUtensorMap xmap, const void* __restrict__ x,
               const float* __restrict__ taps, const uint16_t* __restrict__ w_img,
               void* __restrict__ out, long long n, long long frames, int num_taps,
               int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    constexpr int kSb = sample_bytes(kFmt);
    const Layout lay = chan_layout(num_taps, kSb);
    const int P = lay.P;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_chan_tc;
    const int my_tiles = static_cast<int>(blockIdx.x) < num_tiles
                             ? (num_tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                             : 0;
    const long long full_rows = n / kM;   // rows (frames of 64 samples) the tensor map covers
    auto tile_of = [&](int k) { return static_cast<int>(blockIdx.x) + k * gridDim.x; };
    // First window row of half h of tile k.
    auto row0 = [&](int k, int h) {
        return static_cast<long long>(tile_of(k)) * kFrames + kHalf * h - P;
    };

    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&ctl.full), kWorkerWarps);
        mbar_init(smem_u32(&ctl.empty), 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.win_full[i]), 1);
            mbar_init(smem_u32(&ctl.win_empty[i]), kHalfWarps);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.dfull[i]), 1);
            mbar_init(smem_u32(&ctl.dempty[i]), kWorkerWarps);
        }
        for (int i = 0; i < kExpBufs; ++i) {
            mbar_init(smem_u32(&ctl.eready[i]), kWorkerWarps);
        }
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    __syncthreads();
    if (threadIdx.x == 0 && my_tiles > 0) {
        for (int h = 0; h < 2; ++h) {
            const uint32_t bar = smem_u32(&ctl.win_full[h]);
            mbar_arrive_expect_tx(bar, lay.win);
            tma_load_2d(sbase + lay.win0 + h * lay.win, &xmap, 0, static_cast<int>(row0(0, h)),
                        bar);
        }
    }
    // The twiddle operand (hi and lo, already in the operand layout).
    {
        const uint4* src = reinterpret_cast<const uint4*>(w_img);
        uint4* dst = reinterpret_cast<uint4*>(smem + lay.w_hi);
        for (uint32_t i = threadIdx.x; i < 2 * kSplit / 16; i += kThreads) {
            dst[i] = __ldg(src + i);
        }
        if (kTapsSmem) {
            // taps[p][slot]: slot l < 32 holds branch (64 - l) % 64, slot 32 + l branch 32 - l.
            float* tp = reinterpret_cast<float*>(smem + lay.taps);
            for (int i = threadIdx.x; i < P * kM; i += kThreads) {
                const int pp = i / kM;
                const int slot = i - pp * kM;
                const int m = slot < 32 ? (kM - slot) & (kM - 1) : 32 - (slot - 32);
                const int l = pp * kM + m;
                tp[i] = l < num_taps ? __ldg(taps + l) : 0.0f;
            }
        }
    }
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp < kWorkerWarps) {
        const int wtid = threadIdx.x;
        const int pair = wtid & 31;                      // K indices 2 pair, 2 pair + 1
        const int m_a = k_to_branch(2 * pair);           // their branches
        const int m_b = k_to_branch(2 * pair + 1);
        const uint32_t tap_a = sbase + lay.taps + static_cast<uint32_t>(pair) * 4u;
        const uint32_t tap_b = tap_a + 32u * 4u;
        const int hw = warp / kHalfWarps;                // the half-window this warp reads
        const int fgroup = warp % kHalfWarps;            // frames 8 fgroup .. +7 of half hw
        const int frow0 = kHalf * hw + kR * fgroup;      // their first tile row
        const int quarter = warp & 3;
        const int slice = warp >> 2;                     // channels 16 slice .. +15
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16);

        // Sample s_d of branch m for the thread's frames is x[(t + d) M - m] = window row
        // (t + d - (m > 0)) - r0, column (M - m) % M. `base` addresses d = 0; a block of eight
        // consecutive d is eight loads at fixed offsets. Rows outside the input were
        // zero-filled by the copy; the partial last frame was patched in (patch_partial_row).
        // (The block of the last tap group may start up to 8 rows before the window; those
        // samples are never used and lie in the operand area before it.)
        auto load_block = [&](f32x2 (&blk)[kR], uint32_t base, int d0) {
            const uint32_t a = base + static_cast<uint32_t>(d0 * kM * kSb);
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                blk[i] = lds_sample<kFmt>(a + static_cast<uint32_t>(i * kM * kSb));
            }
        };
        // u[t + i][m] for the thread's 8 frames of one branch m from the warp's half-window.
        auto branch_sums = [&](f32x2 (&acc)[kR], uint32_t buf, int m, uint32_t tap_s) {
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                acc[i] = 0ull;
            }
            // Frame t = first row + P + 8 fgroup; d = 0 is row 8 fgroup + P - (m > 0).
            const uint32_t base =
                buf + static_cast<uint32_t>(((kR * fgroup + P - (m > 0 ? 1 : 0)) * kM +
                                             ((kM - m) & (kM - 1))) * kSb);
            const int groups = P / kR;
            const int rem = P - groups * kR;
            f32x2 a[kR];
            f32x2 b[kR];
            load_block(a, base, 0);
            int g = 0;
            for (; g + 2 <= groups; g += 2) {
                load_block(b, base, -kR * (g + 1));
                branch_group<kTapsSmem>(acc, a, b, taps, tap_s, m, kR * g, kR, num_taps);
                load_block(a, base, -kR * (g + 2));
                branch_group<kTapsSmem>(acc, b, a, taps, tap_s, m, kR * (g + 1), kR, num_taps);
            }
            if (g < groups) {
                load_block(b, base, -kR * (g + 1));
                branch_group<kTapsSmem>(acc, a, b, taps, tap_s, m, kR * g, kR, num_taps);
                if (rem > 0) {
                    load_block(a, base, -kR * (g + 2));
                    branch_group<kTapsSmem>(acc, b, a, taps, tap_s, m, kR * (g + 1), rem, num_taps);
                }
            } else if (rem > 0) {
                load_block(b, base, -kR * (g + 1));
                branch_group<kTapsSmem>(acc, a, b, taps, tap_s, m, kR * g, rem, num_taps);
            }
        };
        // The input's last, partial frame lies outside the tensor map (its copy reads zeros):
        // when a half-window holds that row, the half's warps write its samples in, then sync.
        const int tail = static_cast<int>(n - full_rows * kM);
        const int htid = static_cast<int>(threadIdx.x) - hw * kHalfWarps * 32;
        auto patch_partial_row = [&](uint32_t buf, long long r0) {
            const long long rel = full_rows - r0;
            if (tail == 0 || rel < 0 || rel >= lay.wrows) {
                return;   // uniform across the half's warps
            }
            if (htid < tail) {
                // The stored sample, as the copy would have placed it.
                const uint32_t dst = buf + static_cast<uint32_t>(rel * kM + htid) * kSb;
                const long long s = full_rows * kM + htid;
                if constexpr (kFmt == 0) {
                    const float2 v = __ldg(static_cast<const float2*>(x) + s);
                    sts64(dst, pack2(v.x, v.y));
                } else if constexpr (kFmt == 1) {
                    const uint32_t v = __ldg(static_cast<const unsigned int*>(x) + s);
                    sts32(dst, v);
                } else {
                    const unsigned short v = __ldg(static_cast<const unsigned short*>(x) + s);
                    asm volatile("st.shared.u16 [%0], %1;" ::"r"(dst), "h"(v) : "memory");
                }
            }
            fence_proxy_async_smem();
            asm volatile("bar.sync %0, %1;" ::"r"(1 + hw), "n"(kHalfWarps * 32) : "memory");
        };

        // Branch sums of tile k for this thread: u0 (branch m_a), u1 (m_b), 8 frames.
        f32x2 u0[kR];
        f32x2 u1[kR];
        auto compute = [&](int k) -> bool {
            // Half hw of tile k is the (k + 1)-th fill of buffer hw.
            if (!mbar_wait_bounded(smem_u32(&ctl.win_full[hw]), k & 1, fault, kFaultTileLoad,
                                   abort)) {
                return false;
            }
            const uint32_t buf = sbase + lay.win0 + static_cast<uint32_t>(hw) * lay.win;
            patch_partial_row(buf, row0(k, hw));
            branch_sums(u0, buf, m_a, tap_a);
            branch_sums(u1, buf, m_b, tap_b);
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.win_empty[hw]));
            }
            return true;
        };
        // The A operand of tile k (once the MMAs of tile k - 1 are done), each frame (GEMM row)
        // scaled by its own power of two: the DFT acts on rows, so the drain undoes the scale
        // frame by frame. A warp holds whole frames (all 64 branches of its 8 frames), so a
        // frame's scale is one warp reduction; lane 0 publishes the exponents for the drain.
        auto stage_operand = [&](int k) -> bool {
            int ef[kR];
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                const float2 a = unpack2(u0[i]);
                const float2 b = unpack2(u1[i]);
                // Non-negative floats order like their bit patterns.
                const float m = fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(b.x), fabsf(b.y)));
                // Clamped to 127 (only |u| < 2^-113 would want more): the stored exponent.
                ef[i] = min(scale_exponent(__reduce_max_sync(0xFFFFFFFFu, __float_as_uint(m))),
                            127);
            }
            if (lane == 0) {
                signed char* fe = ctl.fexp[k % kExpBufs];
#pragma unroll
                for (int i = 0; i < kR; ++i) {
                    fe[frow0 + i] = static_cast<signed char>(ef[i]);
                }
                mbar_arrive(smem_u32(&ctl.eready[k % kExpBufs]));
            }
            if (!mbar_wait_bounded(smem_u32(&ctl.empty), (k & 1) ^ 1, fault, kFaultStageEmpty,
                                   abort)) {
                return false;
            }
            const int kre = 2 * pair;
            const int kim = kM + 2 * pair;
            const uint32_t off_re = static_cast<uint32_t>(kre >> 3) * kPlane + (kre & 7) * 2u;
            const uint32_t off_im = static_cast<uint32_t>(kim >> 3) * kPlane + (kim & 7) * 2u;
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                // ef <= 127 and >= -113: 2^ef is one normal float; the scaling is exact.
                const float f = exp2_exact(ef[i]);
                const f32x2 ff = pack2(f, f);
                const float2 a = unpack2(mul2(u0[i], ff));
                const float2 b = unpack2(mul2(u1[i], ff));
                uint32_t re_hi, re_lo, im_hi, im_lo;
                split2(a.x, b.x, re_hi, re_lo);
                split2(a.y, b.y, im_hi, im_lo);
                const uint32_t row = static_cast<uint32_t>(frow0 + i) * 16u;
                sts32(sbase + lay.a_hi + off_re + row, re_hi);
                sts32(sbase + lay.a_lo + off_re + row, re_lo);
                sts32(sbase + lay.a_hi + off_im + row, im_hi);
                sts32(sbase + lay.a_lo + off_im + row, im_lo);
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.full));
            }
            return true;
        };

        bool ok = my_tiles > 0 && compute(0) && stage_operand(0);
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            if (k + 1 < my_tiles && !(compute(k + 1) && stage_operand(k + 1))) {
                break;
            }
            const int db = k & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.dfull[db]), (k >> 1) & 1, fault, kFaultAccumFull,
                                   abort)) {
                break;
            }
            fence_after();
            // v[r]: lanes 32 quarter + 16 r .. + 15 (frames), columns 32 slice .. + 31
            // (channels 16 slice .. + 15, Re and Im), in the 16x256b fragment order.
            float v[2][16];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    v[r][i] = 0.0f;
                }
            }
#pragma unroll
            for (int part = 0; part < kParts; ++part) {
                uint32_t t0[16];
                uint32_t t1[16];
                const uint32_t col =
                    static_cast<uint32_t>((db * kParts + part) * kK + kColsPerSlice * slice);
                tmem_ld_16x256b_x4(lane_addr + col, t0);
                tmem_ld_16x256b_x4(lane_addr + (16u << 16) + col, t1);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    v[0][i] += __uint_as_float(t0[i]);
                    v[1][i] += __uint_as_float(t1[i]);
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.dempty[db]));
            }
            // The frames' exponents (written before the tile's operand, long since complete).
            if (!mbar_wait_bounded(smem_u32(&ctl.eready[k % kExpBufs]), (k / kExpBufs) & 1,
                                   fault, kFaultScale, abort)) {
                break;
            }
            const volatile signed char* fe = ctl.fexp[k % kExpBufs];
            // Four lanes per frame write its channels 16 slice + 8 jj + 2 (lane % 4), + 1: each
            // store fills 64 contiguous bytes of eight frames.
            const long long t_base = static_cast<long long>(tile_of(k)) * kFrames + quarter * 32 +
                                     (lane >> 2);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
#pragma unroll
                for (int s = 0; s < 2; ++s) {
                    const long long t = t_base + 16 * r + 8 * s;
                    // shift in [-141, 99]: 2^shift is one float (subnormal below -126), and the
                    // scaling is exact unless the result itself is subnormal.
                    const float f =
                        exp2_exact(-(fe[quarter * 32 + (lane >> 2) + 16 * r + 8 * s] + kWExp));
                    const f32x2 ff = pack2(f, f);
                    if (t < frames) {
#pragma unroll
                        for (int jj = 0; jj < 2; ++jj) {
                            const float* a = &v[r][4 * (2 * jj) + 2 * s];
                            const float* b = &v[r][4 * (2 * jj + 1) + 2 * s];
                            const long long o = t * kM + 16 * slice + 8 * jj + 2 * (lane & 3);
                            const float2 za = unpack2(mul2(pack2(a[0], a[1]), ff));
                            const float2 zb = unpack2(mul2(pack2(b[0], b[1]), ff));
                            const float re0 = za.x;
                            const float im0 = za.y;
                            const float re1 = zb.x;
                            const float im1 = zb.y;
                            if constexpr (kMag) {
                                // Channels c, c + 1 of the frame: 8 bytes, four lanes 32.
                                *reinterpret_cast<float2*>(static_cast<float*>(out) + o) =
                                    make_float2(cmag(re0, im0), cmag(re1, im1));
                            } else {
                                *reinterpret_cast<float4*>(static_cast<float2*>(out) + o) =
                                    make_float4(re0, im0, re1, im1);
                            }
                        }
                    }
                }
            }
        }
    } else if (warp == kTmaWarp) {
        // Refills half-window h with tile k once every worker warp has read tile k - 1's.
        if (lane == 0) {
            for (int k = 1; k < my_tiles && !*abort; ++k) {
                for (int h = 0; h < 2; ++h) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.win_empty[h]), (k - 1) & 1, fault,
                                           kFaultStageEmpty, abort)) {
                        k = my_tiles;
                        break;
                    }
                    const uint32_t bar = smem_u32(&ctl.win_full[h]);
                    mbar_arrive_expect_tx(bar, lay.win);
                    tma_load_2d(sbase + lay.win0 + static_cast<uint32_t>(h) * lay.win, &xmap, 0,
                                static_cast<int>(row0(k, h)), bar);
                }
            }
        }
    } else if (lane == 0) {
        const uint32_t w_hi = sbase + lay.w_hi;
        const uint32_t w_lo = sbase + lay.w_lo;
        const uint32_t a_hi = sbase + lay.a_hi;
        const uint32_t a_lo = sbase + lay.a_lo;
        for (int k = 0; k < my_tiles && !*abort; ++k) {
            const int db = k & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.full), k & 1, fault, kFaultStageFull, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.dempty[db]), ((k >> 1) & 1) ^ 1, fault,
                                   kFaultAccumEmpty, abort)) {
                break;
            }
            fence_after();
            for (int ks = 0; ks < kK / 16; ++ks) {
                const int steps_per_part = kK / 16 / kParts;
                const uint32_t d =
                    tmem + static_cast<uint32_t>((db * kParts + ks / steps_per_part) * kK);
                const uint32_t off = static_cast<uint32_t>(2 * ks) * kPlane;
                const unsigned long long ah = smem_desc(a_hi + off, kPlane, 128);
                const unsigned long long al = smem_desc(a_lo + off, kPlane, 128);
                const unsigned long long bh = smem_desc(w_hi + off, kPlane, 128);
                const unsigned long long bl = smem_desc(w_lo + off, kPlane, 128);
                mma_f16<kIdesc>(d, ah, bh, (ks % steps_per_part) != 0 ? 1u : 0u);
                mma_f16<kIdesc>(d, ah, bl, 1u);
                mma_f16<kIdesc>(d, al, bh, 1u);
            }
            mma_commit(smem_u32(&ctl.dfull[db]));
            mma_commit(smem_u32(&ctl.empty));
        }
        mma_commit(smem_u32(&ctl.teardown));
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    }
    if (threadIdx.x == 0 && *abort) {
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == kMmaWarp) {
        tmem_dealloc(tmem, kTmemCols);
    }
}

// Builds the twiddle operand image in FP64: B row n (output column), K index k (input
// column), n, k < 128: row n gives part `part` of channel `ch` (column_to_channel); K 0-63
// multiply Re u, 64-127 Im u. Element value 2^14 W split into FP16 hi/lo, stored at the operand layout's offsets.
__global__ void chan_twiddle_kernel(uint16_t* img)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kK * kK) {
        return;
    }
    const int nrow = idx / kK;
    const int kcol = idx % kK;
    int ch = 0;
    int part = 0;
    column_to_channel(nrow, ch, part);
    const int br = k_to_branch(kcol % kM);
    double s, c;
    sincospi(2.0 * static_cast<double>((ch * br) % kM) / kM, &s, &c);
    double v;
    if (part == 0) {
        v = kcol < kM ? c : -s;    // Re z = Re u cos - Im u sin
    } else {
        v = kcol < kM ? s : c;     // Im z = Re u sin + Im u cos
    }
    const float vs = static_cast<float>(v * 16384.0);
    const __half hi = __float2half_rn(vs);
    const __half lo = __float2half_rn(vs - __half2float(hi));
    const uint32_t off = static_cast<uint32_t>(kcol >> 3) * kPlane +
                         static_cast<uint32_t>(nrow) * 16u + static_cast<uint32_t>(kcol & 7) * 2u;
    img[off / 2] = *reinterpret_cast<const uint16_t*>(&hi);
    img[(kSplit + off) / 2] = *reinterpret_cast<const uint16_t*>(&lo);
}

bool chan_tc_supported(int channels, int num_taps)
{
    return channels == kM && num_taps >= 1 && (num_taps + kM - 1) / kM <= kMaxPerBranch &&
           chan_layout(num_taps).bytes <= 227u * 1024u;
}

size_t chan_tc_twiddle_bytes() { return 2 * kSplit; }

cudaError_t chan_tc_build_twiddles(void* img, cudaStream_t stream)
{
    cudaError_t err = cudaMemsetAsync(img, 0, 2 * kSplit, stream);
    if (err != cudaSuccess) {
        return err;
    }
    chan_twiddle_kernel<<<(kK * kK + 255) / 256, 256, 0, stream>>>(static_cast<uint16_t*>(img));
    return cudaGetLastError();
}

template <bool kTapsSmem, bool kMag, int kFmt>
static cudaError_t launch_chan(const void* x, const float* taps, const void* twiddles, void* z,
                               long long n, long long frames, int num_taps, cudaStream_t stream)
{
    const Layout lay = chan_layout(num_taps, sample_bytes(kFmt));
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    cudaFuncAttributes attr{};
    if ((err = cudaFuncGetAttributes(&attr, chan_tc_kernel<kTapsSmem, kMag, kFmt>)) != cudaSuccess) {
        return err;
    }
    if (attr.maxThreadsPerBlock < kThreads) {
        return cudaErrorLaunchOutOfResources;
    }
    err = cudaFuncSetAttribute(chan_tc_kernel<kTapsSmem, kMag, kFmt>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    // x viewed as rows of 128 components (one frame of 64 samples), full frames only; boxes of
    // one half-window. The copy moves the components as stored.
    CUtensorMap map;
    err = encode_rows(&map, x, sample_bytes(kFmt) / 2, n / kM, 2 * kM, 2 * kM,
                      static_cast<uint32_t>(lay.wrows));
    if (err != cudaSuccess) {
        return err;
    }
    const int tiles = static_cast<int>((frames + kFrames - 1) / kFrames);
    const int grid = tiles < sms ? tiles : sms;
    chan_tc_kernel<kTapsSmem, kMag, kFmt><<<grid, kThreads, bytes, stream>>>(
        map, x, taps, static_cast<const uint16_t*>(twiddles),
        z, n, frames, num_taps, tiles);
    return cudaGetLastError();
}

template <int kFmt>
static cudaError_t launch_format(const void* x, const float* taps, const void* twiddles, void* z,
                                 long long n, long long frames, int num_taps, bool magnitude,
                                 cudaStream_t stream)
{
    const bool smem_taps = chan_layout(num_taps).P <= kSmemTapsMax;
    if (magnitude) {
        return smem_taps ? launch_chan<true, true, kFmt>(x, taps, twiddles, z, n, frames,
                                                         num_taps, stream)
                         : launch_chan<false, true, kFmt>(x, taps, twiddles, z, n, frames,
                                                          num_taps, stream);
    }
    return smem_taps
               ? launch_chan<true, false, kFmt>(x, taps, twiddles, z, n, frames, num_taps, stream)
               : launch_chan<false, false, kFmt>(x, taps, twiddles, z, n, frames, num_taps,
                                                 stream);
}

cudaError_t chan_tc_launch(const void* x, const float* taps, const void* twiddles, void* z,
                           long long n, int num_taps, cudaStream_t stream, bool magnitude,
                           int format)
{
    const long long frames = (n + kM - 1) / kM;
    if (frames == 0) {
        return cudaSuccess;
    }
    if (n < kM) {
        return cudaErrorInvalidValue;  // the caller routes inputs shorter than a frame elsewhere
    }
    switch (format) {
    case 0:
        return launch_format<0>(x, taps, twiddles, z, n, frames, num_taps, magnitude, stream);
    case 1:
        return launch_format<1>(x, taps, twiddles, z, n, frames, num_taps, magnitude, stream);
    case 2:
        return launch_format<2>(x, taps, twiddles, z, n, frames, num_taps, magnitude, stream);
    default:
        return cudaErrorInvalidValue;
    }
}

cudaError_t chan_tc_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_chan_tc, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_chan_tc, &zero, sizeof(unsigned int));
}

}  // namespace rfx
