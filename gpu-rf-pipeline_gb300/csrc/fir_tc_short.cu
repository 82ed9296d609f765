// Tensor-core FIR for short filters (2 to 129 taps) on sm_103a: the block-Toeplitz GEMM of
// fir_tc.cu, re-tiled so that each sample crosses HBM and the copy engine once.
//
//   y[n] = sum_{k<K} h[k] x[n-k],  x[m < 0] = 0                              (src/fir.cu:1-5)
//
// With blocks of B = 128 outputs and K <= 129 a block reaches back one block (C = 1):
//   Y[:, j] = T_0 X[:, j] + T_1 X[:, j - 1],   T_c(r, s) = h[cB + r - s]  (0 outside [0, K)).
// A tile is NB = 48 blocks (6144 outputs); its input window is blocks j0 - 1 .. j0 + 47 (49
// rows of 128 samples). The GEMM per tile is D (128 x 96) += A (128 x 16) B (16 x 96) over
// K-steps (c, st): A is a descriptor into the tap strip (fir_tc.cu's layout: output rows stored
// reversed, so every 8 x 8 core matrix of T_0, T_1 is one strip element), B the FP16 planes of
// K-step st (16 samples of each window row, N index 2 j + {0: I, 1: Q}); chunk 1 of a K-step
// whose taps are all zero (16 st <= 113 - K) is skipped: 63 taps need 12 of the 16 chunk-steps.
//
// What differs from fir_tc.cu, which serves long filters:
//  * the whole window arrives by ONE 2-D TMA copy (49 rows of 1 KB for cf32) into a ring of
//    three window buffers, issued by a copy warp as soon as a buffer is converted: each sample
//    crosses HBM once and the TMA engine once (fir_tc.cu copies it twice: a scan slice and a
//    K-step box). A window is held from its copy until its tile is converted, and under full
//    load a 50-64 KB copy takes about 7 us to land, so two buffers left the tile period at half
//    of (copy + scan + conversion), about 4.5 us; three bring it to the HBM rate (measured: a
//    plain TMA stream through two 64 KB buffers per SM moves 5.5 TB/s);
//  * the tile's power-of-two scale (largest |component| of the window brought into
//    [2^14, 2^15)) is a scan of that resident window by four scan warps as soon as it lands;
//    the eight producer warps only convert, from the same buffer, and have no copy duties;
//  * one accumulation group per tile: H (h_hi x_hi, at most 16 MMAs) and X (the two cross
//    products) in two TMEM buffers of 256 columns each, so the MMAs of tile k + 1 run while
//    eight drain warps read tile k, add H + X, scale by 2^-(ex + eh) and store.
// Split precision as in fir_tc.cu: x' = 2^ex x = x_hi + x_lo, h' = 2^eh h = h_hi + h_lo in FP16;
// the MMAs sum h_hi x_hi + h_hi x_lo + h_lo x_hi with FP32 accumulation.
//
// Roles (704 threads): warp 0 copies windows; warp 1 owns tensor memory and issues the MMAs (the
// warp runs the loop, one elected lane issues); warps 2-9 produce (FP16 hi/lo planes); warps
// 10-17 drain (warp w reads TMEM lane quarter w % 4, the columns of blocks 24 h .. 24 h + 23
// with h = (w - 10) / 4); warps 18-21 scan windows. Every wait is an mbarrier wait bounded in
// time, polled by every lane of a waiting warp (measured: lane 0 polling alone and handing the
// result to the warp by a shuffle took 18 us longer at 63 taps, the hand-off latency landing on
// every K-step); a give-up sets the fault word and every role stops.
#include "fir_tc.cuh"
#include "sample_fmt.cuh"
#include "tc_common.cuh"
#include "tmap.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_fir_tcs;

namespace {

using namespace tc;

constexpr int kB = 128;                   // outputs per block = MMA M
constexpr int kNB = 48;                   // blocks per tile; MMA N = 2 * kNB
constexpr int kWinBufs = 3;               // tile windows resident or in flight
constexpr int kN = 2 * kNB;
constexpr int kC = 1;                     // previous blocks a block reaches back to
constexpr int kRows = kNB + kC;           // window rows per tile
constexpr int kSteps = kB / 16;           // K-steps of 16 samples per tile
constexpr int kS = 8;                     // operand stages
constexpr int kGroup = 4;                 // K-steps the producers convert at once
static_assert(kS % kGroup == 0 && kSteps % kGroup == 0, "producer groups");
constexpr int kCopyWarp = 0;
constexpr int kMmaWarp = 1;
constexpr int kFirstProducerWarp = 2;
constexpr int kProducerWarps = 8;
constexpr int kProducers = kProducerWarps * 32;
constexpr int kFirstDrainWarp = kFirstProducerWarp + kProducerWarps;
constexpr int kDrainWarps = 8;
constexpr int kFirstScanWarp = kFirstDrainWarp + kDrainWarps;
constexpr int kScanWarps = 4;
constexpr int kThreads = (kFirstScanWarp + kScanWarps) * 32;
constexpr int kScales = 8;                // tile scales published ahead (ring)
constexpr uint32_t kTmemCols = 512;       // 2 tiles x (H: kN columns, X: kN columns), 384 used
constexpr uint32_t kIdesc = idesc_f16(kB, kN);
constexpr int kTapCores = 16 * kC + 31;   // core matrices of the tap strip
constexpr uint32_t kPitch = 2u * kRows * 16u + 16u;   // bytes per plane (+16: banks)
constexpr uint32_t kSplit = 2u * kPitch;              // one split (hi or lo): 2 planes
constexpr uint32_t kStage = 2u * kSplit;              // one operand stage: hi + lo
constexpr uint32_t kTapsHi = 1024;
constexpr uint32_t kTapsLo = kTapsHi + 128u * kTapCores;
constexpr uint32_t kStages0 = (kTapsLo + 128u * kTapCores + 1023u) & ~1023u;
constexpr uint32_t kWin0 = (kStages0 + kS * kStage + 1023u) & ~1023u;
// A group's items (K-step g, row b, sample pair q), numbered f = (g kRows + b) 8 + q, are
// dealt to the producer threads in turn: thread t takes f = t, t + kProducers, ... (q = t % 8
// throughout, so eight consecutive lanes write one 16-byte plane row each: no bank conflicts).
constexpr int kGroupItems = kGroup * kRows * 8;
constexpr int kItemIters = (kGroupItems + kProducers - 1) / kProducers;

// Bytes of one window buffer for components of es bytes (256 components per row).
__host__ __device__ constexpr uint32_t win_bytes(int es)
{
    return static_cast<uint32_t>(kRows) * 256u * static_cast<uint32_t>(es);
}

struct Ctrl {
    unsigned long long full[kS];      // stage converted (every producer warp)
    unsigned long long empty[kS];     // stage read by its MMAs (tcgen05.commit)
    unsigned long long win_full[kWinBufs];   // window copied (transaction bytes)
    unsigned long long win_empty[kWinBufs];  // window converted (every producer warp)
    unsigned long long tfull[2];      // a tile's H and X summed (tcgen05.commit)
    unsigned long long tempty[2];     // H and X read (every drain warp)
    unsigned long long sready[kScales];  // the scale of tile k is in ex[k % kScales]
    unsigned long long pready[2];     // every scan warp's part of a window's maximum written
    unsigned long long patched;       // the partial last block written into its window row
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t pmax[2][kScanWarps];
    int ex[kScales];
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");
static_assert(kNB % 16 == 0, "a drain warp reads its kNB columns of H and X 16 at a time");

}  // namespace

// wmap: x as rows of 256 components (one 128-sample block per row, full blocks only), boxes
// of 256 components x kRows rows (one tile window). kFmt: 0 cf32, 1 ci16, 2 ci8 (the copy moves
// the components as stored; the producers decode them).
template <int kFmt>
__global__ void __launch_bounds__(kThreads, 1)
fir_tcs_kernel(const __grid_constant__ CUtensorMap wmap, const void* __restrict__ x,
               const float* __restrict__ taps, float2* __restrict__ y, long long n, int num_taps,
               int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    constexpr int es = component_bytes(kFmt);
    constexpr uint32_t kWin = win_bytes(es);
    constexpr uint32_t kPairBytes = 4u * es;   // two samples as stored
    // The warp index through a shuffle: provably the same on every lane of a warp, so values
    // derived from it in a role's loop can stay in uniform registers.
    const int warp = __shfl_sync(0xFFFFFFFFu, static_cast<int>(threadIdx.x >> 5), 0);
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_tcs;
    const int my_tiles = static_cast<int>(blockIdx.x) < num_tiles
                             ? (num_tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                             : 0;
    const long long full_blocks = n / kB;      // rows the tensor map covers
    auto tile_of = [&](int k) { return static_cast<long long>(blockIdx.x) + static_cast<long long>(k) * gridDim.x; };
    auto issue_window = [&](int k) {
        const uint32_t bar = smem_u32(&ctl.win_full[k % kWinBufs]);
        mbar_arrive_expect_tx(bar, kWin);
        tma_load_2d(sbase + kWin0 + static_cast<uint32_t>(k % kWinBufs) * kWin, &wmap, 0,
                    static_cast<int>(tile_of(k) * kNB - kC), bar);
    };

    // ---- setup: barriers, tensor memory, the first window, tap strip -----------------------
    if (threadIdx.x == 0) {
        for (int i = 0; i < kS; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < kWinBufs; ++i) {
            mbar_init(smem_u32(&ctl.win_full[i]), 1);
            mbar_init(smem_u32(&ctl.win_empty[i]), kProducerWarps);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.tfull[i]), 1);
            mbar_init(smem_u32(&ctl.tempty[i]), kDrainWarps);
        }
        for (int i = 0; i < kScales; ++i) {
            mbar_init(smem_u32(&ctl.sready[i]), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.pready[i]), kScanWarps);
        }
        mbar_init(smem_u32(&ctl.patched), kScanWarps);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        ctl.tap_max = 0;
        fence_mbar_init();
        for (int k = 0; k < kWinBufs && k < my_tiles; ++k) {
            issue_window(k);   // thread 0 is the copy warp's issuing lane
        }
    }
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    // Largest tap magnitude (bit pattern of |h|: ordered like the value).
    {
        uint32_t m = 0;
        for (int k = threadIdx.x; k < num_taps; k += kThreads) {
            m = max(m, absbits(__ldg(taps + k)));
        }
        m = __reduce_max_sync(0xFFFFFFFFu, m);
        __syncthreads();   // tap_max initialised
        if (lane == 0 && m != 0) {
            atomicMax(&ctl.tap_max, m);
        }
    }
    __syncthreads();
    const int eh = scale_exponent(ctl.tap_max);
    {
        // The strip G[t][q][e] = 2^eh h[(C + 1) B - 1 - 8 t - q - e], FP16 hi and lo: two
        // adjacent elements e, e + 1 of core matrix t, row q per iteration.
        const float fa = exp2i(eh / 2);
        const float fb = exp2i(eh - eh / 2);
        const int dmax = (kC + 1) * kB - 1;
        for (int i = threadIdx.x; i < kTapCores * 32; i += kThreads) {
            const int t = i >> 5;
            const int q = (i >> 2) & 7;
            const int e = (i & 3) * 2;
            const int i0 = dmax - 8 * t - q - e;
            const int i1 = i0 - 1;
            const float v0 = (i0 >= 0 && i0 < num_taps) ? __ldg(taps + i0) * fa * fb : 0.0f;
            const float v1 = (i1 >= 0 && i1 < num_taps) ? __ldg(taps + i1) * fa * fb : 0.0f;
            uint32_t hi, lo;
            split2(v0, v1, hi, lo);
            const uint32_t off = static_cast<uint32_t>(t) * 128u + q * 16u + e * 2u;
            sts32(sbase + kTapsHi + off, hi);
            sts32(sbase + kTapsLo + off, lo);
        }
    }
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp == kCopyWarp) {
        // ---- copies: window k once every producer has converted tile k - kWinBufs ---------
        if (lane == 0) {
            for (int k = kWinBufs; k < my_tiles && !*abort; ++k) {
                if (!mbar_wait_bounded(smem_u32(&ctl.win_empty[k % kWinBufs]),
                                       ((k / kWinBufs) & 1) ^ 1, fault, kFaultStageEmpty, abort)) {
                    break;
                }
                issue_window(k);
            }
        }
    } else if (warp == kMmaWarp) {
        // ---- MMA issuer: the whole warp runs the loop, one elected lane issues -------------
        // Chunk 1 of K-step st holds taps only from 16 st > 113 - K on.
        const int st_c1 = num_taps >= 114 ? 0 : (113 - num_taps) / 16 + 1;
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, kPitch, 128);
        // Start-address fields (address / 16): chunk 0 of K-step st starts 16 C + 2 st strip
        // elements in and C blocks (2 C plane rows) into the stage; chunk 1 is 16 strip
        // elements (128 units) and 2 rows (2 units) lower.
        const uint32_t a_hi0 = ((sbase + kTapsHi) >> 4) + static_cast<uint32_t>(16 * kC) * 8u;
        const uint32_t a_lo0 = ((sbase + kTapsLo) >> 4) + static_cast<uint32_t>(16 * kC) * 8u;
        const uint32_t b_base = ((sbase + kStages0) >> 4) + static_cast<uint32_t>(2 * kC);
        bool stop = false;
        int u = 0;   // K-steps issued (block-wide numbering)
        for (int k = 0; k < my_tiles && !stop && !*abort; ++k) {
            const int buf = k & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.tempty[buf]), ((k >> 1) & 1) ^ 1, fault,
                                        kFaultAccumEmpty, abort)) {
                break;
            }
            fence_after();
            const uint32_t h_acc = tmem + static_cast<uint32_t>(buf) * (2u * kN);
            const uint32_t x_acc = h_acc + kN;
            for (int st = 0; st < kSteps; ++st, ++u) {
                const int slot = u % kS;
                if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (u / kS) & 1, fault,
                                            kFaultStageFull, abort)) {
                    stop = true;
                    break;
                }
                fence_after();
                const uint32_t off = static_cast<uint32_t>(2 * st) * 8u;
                const unsigned long long dah = a_desc | (a_hi0 + off);
                const unsigned long long dal = a_desc | (a_lo0 + off);
                const unsigned long long dbh =
                    b_desc | (b_base + static_cast<uint32_t>(slot) * (kStage >> 4));
                const unsigned long long dbl = dbh + (kSplit >> 4);
                const uint32_t acc = st > 0 ? 1u : 0u;
                const bool chunk1 = st >= st_c1;
                if (elect_one()) {
                    mma_f16<kIdesc>(h_acc, dah, dbh, acc);
                    mma_f16<kIdesc>(x_acc, dah, dbl, acc);
                    mma_f16_acc<kIdesc>(x_acc, dal, dbh);
                    if (chunk1) {
                        mma_f16_acc<kIdesc>(h_acc, dah - 128, dbh - 2);
                        mma_f16_acc<kIdesc>(x_acc, dah - 128, dbl - 2);
                        mma_f16_acc<kIdesc>(x_acc, dal - 128, dbh - 2);
                    }
                    mma_commit(smem_u32(&ctl.empty[slot]));
                }
                __syncwarp();
            }
            if (!stop && elect_one()) {
                mma_commit(smem_u32(&ctl.tfull[buf]));
            }
            __syncwarp();
        }
        // Every MMA the elected lane issued has completed before tensor memory is released.
        if (elect_one()) {
            mma_commit(smem_u32(&ctl.teardown));
        }
        __syncwarp();
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    } else if (warp < kFirstDrainWarp) {
        // ---- producers: the FP16 planes of each K-step ------------------------------------
        const int ptid = static_cast<int>(threadIdx.x) - kFirstProducerWarp * 32;
        const int q = ptid & 7;
        const uint32_t elem_off = static_cast<uint32_t>(q >> 2) * kPitch +
                                  static_cast<uint32_t>(q & 3) * 4u;
        // The thread's items are at the same places in every group: window offset (K-step
        // g of the group, row b, pair q) relative to the group's first K-step, and plane offset
        // relative to the group's first stage. The group's stages are consecutive slots (kS is
        // a multiple of kGroup). ~0 marks an unused item.
        uint32_t src_off[kItemIters];
        uint32_t dst_off[kItemIters];
#pragma unroll
        for (int i = 0; i < kItemIters; ++i) {
            const int f8 = (ptid >> 3) + (kProducers / 8) * i;   // g kRows + b
            const int g = f8 / kRows;
            const int b = f8 - g * kRows;
            src_off[i] = f8 < kGroup * kRows
                             ? static_cast<uint32_t>(b * 128 + 16 * g + 2 * q) * (kPairBytes / 2)
                             : ~0u;
            dst_off[i] = static_cast<uint32_t>(g) * kStage + elem_off +
                         static_cast<uint32_t>(2 * b) * 16u;
        }
        int u = 0;
        bool ok = true;
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            const int wb = k % kWinBufs;
            // The tile's scale (published by the scan warps once they scanned the window,
            // partial block included) and its window.
            if (!mbar_wait_bounded(smem_u32(&ctl.sready[k % kScales]), (k / kScales) & 1,
                                        fault, kFaultScale, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.win_full[wb]), (k / kWinBufs) & 1, fault,
                                        kFaultTileLoad, abort)) {
                break;
            }
            const uint32_t win = sbase + kWin0 + static_cast<uint32_t>(wb) * kWin;
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k % kScales]);
            const float fs = exp2_exact(ex);
            const f32x2 fs2 = pack2(fs, fs);
            // K-steps in groups of kGroup: a thread's items of the whole group are independent,
            // so their loads, splits and stores overlap, and the group takes one proxy fence.
            for (int st0 = 0; st0 < kSteps && ok; st0 += kGroup, u += kGroup) {
#pragma unroll
                for (int g = 0; g < kGroup; ++g) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.empty[(u + g) % kS]),
                                           (((u + g) / kS) & 1) ^ 1, fault, kFaultStageEmpty,
                                           abort)) {
                        ok = false;
                    }
                }
                if (!ok) {
                    break;
                }
                const uint32_t src0 =
                    win + static_cast<uint32_t>(16 * st0) * (kPairBytes / 2);
                const uint32_t dst0 = sbase + kStages0 + static_cast<uint32_t>(u % kS) * kStage;
#pragma unroll
                for (int i = 0; i < kItemIters; ++i) {
                    if (src_off[i] != ~0u) {
                        const float4 v4 = lds_pair(src0 + src_off[i], kFmt);
                        const float2 s0 = unpack2(mul2(pack2(v4.x, v4.y), fs2));
                        const float2 s1 = unpack2(mul2(pack2(v4.z, v4.w), fs2));
                        uint32_t re_hi, re_lo, im_hi, im_lo;
                        split2(s0.x, s1.x, re_hi, re_lo);
                        split2(s0.y, s1.y, im_hi, im_lo);
                        const uint32_t row_re = dst0 + dst_off[i];
                        sts32(row_re, re_hi);
                        sts32(row_re + 16u, im_hi);
                        sts32(row_re + kSplit, re_lo);
                        sts32(row_re + kSplit + 16u, im_lo);
                    }
                }
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
#pragma unroll
                    for (int g = 0; g < kGroup; ++g) {
                        mbar_arrive(smem_u32(&ctl.full[(u + g) % kS]));
                    }
                }
            }
            if (!ok) {
                break;
            }
            // Every K-step of the tile is converted: the window may be refilled.
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.win_empty[wb]));
            }
        }
    } else if (warp < kFirstScanWarp) {
        // ---- drain warps: H + X, scaled, stored ---------------------------------------------
        const int quarter = warp & 3;
        const int half = (warp - kFirstDrainWarp) >> 2;        // blocks kNB/2 half .. + kNB/2 - 1
        const int r = kB - 1 - (quarter * 32 + lane);          // output row of this TMEM lane
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(half * kNB);
        for (int k = 0; k < my_tiles && !*abort; ++k) {
            const int buf = k & 1;
            // The scale ring holds kScales tiles: tile k + 8's window lands only after the
            // producers converted tile k + 5, which needed the MMAs of tile k + 5, which needed
            // tile k + 3 drained: ex[k % kScales] is read before it is rewritten.
            if (!mbar_wait_bounded(smem_u32(&ctl.tfull[buf]), (k >> 1) & 1, fault,
                                        kFaultAccumFull, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.sready[k % kScales]), (k / kScales) & 1,
                                        fault, kFaultScale, abort)) {
                break;
            }
            fence_after();
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k % kScales]);
            const int shift = -(ex + eh);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            const long long jb0 = tile_of(k) * kNB + half * (kNB / 2);
            const uint32_t col0 = static_cast<uint32_t>(buf) * (2u * kN);
#pragma unroll
            for (int c16 = 0; c16 < kNB / 16; ++c16) {
                uint32_t th[16];
                uint32_t tx[16];
                tmem_ld16(lane_addr + col0 + static_cast<uint32_t>(c16 * 16), th);
                tmem_ld16(lane_addr + col0 + kN + static_cast<uint32_t>(c16 * 16), tx);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const long long o = (jb0 + c16 * 8 + i) * kB + r;
                    if (o < n) {
                        const float re = __uint_as_float(th[2 * i]) + __uint_as_float(tx[2 * i]);
                        const float im =
                            __uint_as_float(th[2 * i + 1]) + __uint_as_float(tx[2 * i + 1]);
                        y[o] = make_float2(re * fa * fb, im * fa * fb);
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.tempty[buf]));
            }
        }
    } else {
        // ---- scan warps: each window's scale as soon as it lands ----------------------------
        // The largest |component| of the window brought into [2^14, 2^15), clamped to 127 so
        // that 2^ex is one float and the scaling one exact multiply, published to the producers
        // and the drain warps. A separate role, so that a scale never waits behind a drain.
        const int sw = warp - kFirstScanWarp;
        const int stid = static_cast<int>(threadIdx.x) - kFirstScanWarp * 32;
        const int tail = static_cast<int>(n - full_blocks * kB);   // samples of a partial block
        for (int j = 0; j < my_tiles && !*abort; ++j) {
            const int wb = j % kWinBufs;
            if (!mbar_wait_bounded(smem_u32(&ctl.win_full[wb]), (j / kWinBufs) & 1, fault,
                                        kFaultTileLoad, abort)) {
                break;
            }
            const uint32_t win = sbase + kWin0 + static_cast<uint32_t>(wb) * kWin;
            // The input's last, partial block lies outside the tensor map (its copy read
            // zeros): its stored samples go into their window row (only one tile of a block
            // holds that row), then the scan warps wait for each other.
            const long long rel = full_blocks - (tile_of(j) * kNB - kC);
            if (tail > 0 && rel >= 0 && rel < kRows) {   // uniform across the scan warps
                const uint32_t row = win + static_cast<uint32_t>(rel) * 256u * es;
                for (int i = stid; i < tail; i += kScanWarps * 32) {
                    const long long sidx = full_blocks * kB + i;
                    if constexpr (kFmt == 0) {
                        const float2 v = __ldg(static_cast<const float2*>(x) + sidx);
                        sts64(row + static_cast<uint32_t>(i) * 8u, pack2(v.x, v.y));
                    } else if constexpr (kFmt == 1) {
                        sts32(row + static_cast<uint32_t>(i) * 4u,
                              __ldg(static_cast<const unsigned int*>(x) + sidx));
                    } else {
                        const unsigned short v = __ldg(static_cast<const unsigned short*>(x) + sidx);
                        asm volatile("st.shared.u16 [%0], %1;"
                                     ::"r"(row + static_cast<uint32_t>(i) * 2u), "h"(v)
                                     : "memory");
                    }
                }
                // The window is refilled by TMA later: order these writes before that.
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.patched));
                }
                if (!mbar_wait_bounded(smem_u32(&ctl.patched), 0, fault, kFaultTileLoad,
                                            abort)) {
                    break;
                }
            }
            uint32_t m = 0;
            constexpr int kPairs = kRows * 64;
#pragma unroll 4
            for (int f = stid; f < kPairs; f += kScanWarps * 32) {
                m = max(m, absmax4(lds_pair(win + static_cast<uint32_t>(f) * kPairBytes, kFmt)));
            }
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            // (Two maximum buffers suffice: a warp writes tile j + 2's only after every warp has
            // arrived for tile j + 1, i.e. after it read tile j's.)
            if (lane == 0) {
                ctl.pmax[j & 1][sw] = m;
                mbar_arrive(smem_u32(&ctl.pready[j & 1]));
            }
            if (!mbar_wait_bounded(smem_u32(&ctl.pready[j & 1]), (j >> 1) & 1, fault,
                                        kFaultScale, abort)) {
                break;
            }
            uint32_t tmax = 0;
#pragma unroll
            for (int w = 0; w < kScanWarps; ++w) {
                tmax = max(tmax, *reinterpret_cast<volatile uint32_t*>(&ctl.pmax[j & 1][w]));
            }
            if (stid == 0) {
                ctl.ex[j % kScales] = min(scale_exponent(tmax), 127);
                mbar_arrive(smem_u32(&ctl.sready[j % kScales]));
            }
        }
    }

    // After a give-up, TMA copies may still be in flight: give them time to land (bounded).
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

bool fir_tcs_supported(int num_taps) { return num_taps >= 2 && num_taps <= kC * kB + 1; }

long long fir_tcs_tile_outputs() { return static_cast<long long>(kNB) * kB; }

template <int kFmt>
static cudaError_t launch_tcs(const void* x, const float* taps, void* y, long long n, int num_taps,
                              cudaStream_t stream)
{
    constexpr int es = component_bytes(kFmt);
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
    uint32_t bytes = kWin0 + kWinBufs * win_bytes(es);
    bytes = bytes > 120u * 1024u ? bytes : 120u * 1024u;
    if (bytes > static_cast<uint32_t>(optin)) {
        return cudaErrorInvalidValue;
    }
    err = cudaFuncSetAttribute(fir_tcs_kernel<kFmt>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    // x as rows of 256 components (one 128-sample block per row), full blocks only; one box
    // is a tile window of kRows rows.
    CUtensorMap map;
    err = encode_rows(&map, x, es, n / kB, 2 * kB, 2 * kB, static_cast<uint32_t>(kRows));
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + kB - 1) / kB;
    const int tiles = static_cast<int>((blocks + kNB - 1) / kNB);
    const int grid = tiles < sms ? tiles : sms;
    fir_tcs_kernel<kFmt><<<grid, kThreads, bytes, stream>>>(map, x, taps,
                                                           static_cast<float2*>(y), n, num_taps,
                                                           tiles);
    return cudaGetLastError();
}

cudaError_t fir_tcs_launch(int format, const void* x, const float* taps, void* y, long long n,
                           int num_taps, cudaStream_t stream)
{
    if (n < kB || !fir_tcs_supported(num_taps)) {
        return cudaErrorInvalidValue;
    }
    switch (format) {
    case 0:
        return launch_tcs<0>(x, taps, y, n, num_taps, stream);
    case 1:
        return launch_tcs<1>(x, taps, y, n, num_taps, stream);
    case 2:
        return launch_tcs<2>(x, taps, y, n, num_taps, stream);
    default:
        return cudaErrorInvalidValue;
    }
}

cudaError_t fir_tcs_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_tcs, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_tcs, &zero, sizeof(unsigned int));
}

}  // namespace rfx
