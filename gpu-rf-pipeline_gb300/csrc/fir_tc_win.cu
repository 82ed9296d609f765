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
// Roles (640 threads): warp 0 copies windows; warp 1 owns tensor memory and issues the MMAs (the
// warp runs the loop, one elected lane issues); warps 2-9 produce (FP16 hi/lo planes); warps
// 10-17 drain (warp w reads TMEM lane quarter w % 4, the columns of blocks 24 h .. 24 h + 23
// with h = (w - 10) / 4); warps 18-19 scan windows. Every wait is an mbarrier wait bounded in
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

static __device__ unsigned int g_fault_fir_tcw;

namespace {

using namespace tc;

constexpr int kB = 128;                   // outputs per block = MMA M
constexpr int kNB = 48;                   // blocks per tile; MMA N = 2 * kNB
constexpr int kN = 2 * kNB;
constexpr int kCMax = 3;                  // blocks a block reaches back to, at most (385 taps)
constexpr int kRowsMax = kNB + kCMax;     // window rows per tile, at most
constexpr int kSteps = kB / 16;           // K-steps of 16 samples per tile
constexpr int kStages = 8;                // operand stages
constexpr int kWins = 3;                  // window buffers
constexpr int kGroup = 4;                 // K-steps the producers convert at once
constexpr int kHGroup = 18;               // MMAs per H accumulation, at most
constexpr int kScales = 8;                // tile scales published ahead (ring)
constexpr int kCopyWarp = 0;
constexpr int kMmaWarp = 1;
constexpr int kFirstProducerWarp = 2;
constexpr int kProducerWarps = 8;
constexpr int kProducers = kProducerWarps * 32;
constexpr int kFirstDrainWarp = kFirstProducerWarp + kProducerWarps;
constexpr int kDrainWarps = 8;
constexpr int kFirstScanWarp = kFirstDrainWarp + kDrainWarps;
constexpr int kScanWarps = 2;
constexpr int kThreads = (kFirstScanWarp + kScanWarps) * 32;
constexpr uint32_t kTmemCols = 512;       // H0, H1, X0, X1 of kN columns each: 384 used
constexpr uint32_t kXCol = 2 * kN;        // first column of X0
constexpr uint32_t kIdesc = idesc_f16(kB, kN);
// A group's items (K-step g, row b, sample pair q), numbered f = (g rows + b) 8 + q, are dealt
// to the producer threads in turn: thread t takes f = t, t + kProducers, ... (q = t % 8
// throughout, so eight consecutive lanes write one 16-byte plane row each: no bank conflicts).
constexpr int kItemIters = (kGroup * kRowsMax * 8 + kProducers - 1) / kProducers;
static_assert(kNB % 16 == 0, "a drain warp reads its kNB columns 16 at a time");
static_assert(kSteps % kGroup == 0, "producer groups");

// Shared-memory layout of one launch (C, window buffers, stages and the sample format fixed).
struct Layout {
    int C;               // blocks a block reaches back to
    int rows;            // window rows: kNB + C
    int wins;            // window buffers (2 or 3)
    int stages;          // operand stages (4 or 8)
    int tcount;          // core matrices of the tap strip: 16 C + 31
    uint32_t pitch;      // bytes per plane: 2 rows x 16 B per block + 16 (banks)
    uint32_t split;      // one split (hi or lo) of a stage: 2 planes
    uint32_t stage;      // one operand stage: hi + lo
    uint32_t win;        // one window buffer: rows x 256 components
    uint32_t taps_hi, taps_lo, stages0, win0, bytes;
};

__host__ __device__ inline Layout win_layout(int num_taps, int wins, int stages, int es)
{
    Layout l;
    l.C = (num_taps + kB - 2) / kB;
    l.rows = kNB + l.C;
    l.wins = wins;
    l.stages = stages;
    l.tcount = 16 * l.C + 31;
    l.pitch = static_cast<uint32_t>(2 * l.rows) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    l.win = static_cast<uint32_t>(l.rows) * 256u * static_cast<uint32_t>(es);
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount);
    l.stages0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount) + 1023u) & ~1023u;
    l.win0 = (l.stages0 + static_cast<uint32_t>(stages) * l.stage + 1023u) & ~1023u;
    l.bytes = l.win0 + static_cast<uint32_t>(wins) * l.win;
    return l;
}

struct Ctrl {
    unsigned long long full[kStages];    // stage converted (every producer warp)
    unsigned long long empty[kStages];   // stage read by its MMAs (tcgen05.commit)
    unsigned long long win_full[kWins];  // window copied (transaction bytes)
    unsigned long long win_empty[kWins]; // window converted (every producer warp)
    unsigned long long hfull[2];         // an H group summed (tcgen05.commit)
    unsigned long long hempty[2];        // an H group read (every drain warp)
    unsigned long long xfull[2];         // a tile's X summed (tcgen05.commit)
    unsigned long long xempty[2];        // a tile's X read (every drain warp)
    unsigned long long sready[kScales];  // the scale of tile k is in ex[k % kScales]
    unsigned long long pready[2];        // every scan warp's part of a window's maximum written
    unsigned long long patched;          // the partial last block written into its window row
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t pmax[2][kScanWarps];
    int ex[kScales];
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

}  // namespace

// wmap: x as rows of 256 components (one 128-sample block per row, full blocks only), boxes
// of 256 components x `rows` rows (one tile window). kFmt: 0 cf32, 1 ci16, 2 ci8 (the copy
// moves the components as stored; the producers decode them).
template <int C, int kFmt>
__global__ void __launch_bounds__(kThreads, 1)
fir_tcw_kernel(const __grid_constant__ CUtensorMap wmap, const void* __restrict__ x,
               const float* __restrict__ taps, float2* __restrict__ y, long long n, int num_taps,
               int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    constexpr int es = component_bytes(kFmt);
    constexpr uint32_t kPairBytes = 4u * es;   // two samples as stored
    constexpr int rows = kNB + C;
    constexpr int hks = kSteps < kHGroup / (C + 1) ? kSteps : kHGroup / (C + 1);
    constexpr int groups = (kSteps + hks - 1) / hks;
    static_assert(hks >= 1, "an H group holds at least one K-step");
    constexpr int wins = kWins;
    constexpr int stages = kStages;
    const Layout lay = win_layout(C * kB, wins, stages, es);
    // The warp index through a shuffle: provably the same on every lane of a warp, so values
    // derived from it in a role's loop can stay in uniform registers.
    const int warp = __shfl_sync(0xFFFFFFFFu, static_cast<int>(threadIdx.x >> 5), 0);
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_tcw;
    const int my_tiles = static_cast<int>(blockIdx.x) < num_tiles
                             ? (num_tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                             : 0;
    const long long full_blocks = n / kB;      // rows the tensor map covers
    // H groups: hks whole K-steps of at most kHGroup MMAs each (a K-step issues C + 1).
    auto tile_of = [&](int k) {
        return static_cast<long long>(blockIdx.x) + static_cast<long long>(k) * gridDim.x;
    };
    auto issue_window = [&](int k) {
        const uint32_t bar = smem_u32(&ctl.win_full[k % wins]);
        mbar_arrive_expect_tx(bar, lay.win);
        tma_load_2d(sbase + lay.win0 + static_cast<uint32_t>(k % wins) * lay.win, &wmap, 0,
                    static_cast<int>(tile_of(k) * kNB - C), bar);
    };

    // ---- setup: barriers, tensor memory, the first windows, tap strip ----------------------
    if (threadIdx.x == 0) {
        for (int i = 0; i < stages; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < wins; ++i) {
            mbar_init(smem_u32(&ctl.win_full[i]), 1);
            mbar_init(smem_u32(&ctl.win_empty[i]), kProducerWarps);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.hfull[i]), 1);
            mbar_init(smem_u32(&ctl.hempty[i]), kDrainWarps);
            mbar_init(smem_u32(&ctl.xfull[i]), 1);
            mbar_init(smem_u32(&ctl.xempty[i]), kDrainWarps);
            mbar_init(smem_u32(&ctl.pready[i]), kScanWarps);
        }
        for (int i = 0; i < kScales; ++i) {
            mbar_init(smem_u32(&ctl.sready[i]), 1);
        }
        mbar_init(smem_u32(&ctl.patched), kScanWarps);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        ctl.tap_max = 0;
        fence_mbar_init();
        for (int k = 0; k < wins && k < my_tiles; ++k) {
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
        const int dmax = (C + 1) * kB - 1;
        for (int i = threadIdx.x; i < lay.tcount * 32; i += kThreads) {
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
            sts32(sbase + lay.taps_hi + off, hi);
            sts32(sbase + lay.taps_lo + off, lo);
        }
    }
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp == kCopyWarp) {
        // ---- copies: window k once every producer has converted tile k - wins ---------------
        if (lane == 0) {
            for (int k = wins; k < my_tiles && !*abort; ++k) {
                if (!mbar_wait_bounded(smem_u32(&ctl.win_empty[k % wins]), ((k / wins) & 1) ^ 1,
                                       fault, kFaultStageEmpty, abort)) {
                    break;
                }
                issue_window(k);
            }
        }
    } else if (warp == kMmaWarp) {
        // ---- MMA issuer: the whole warp runs the loop, one elected lane issues -------------
        // Chunk C of K-step st holds taps only from 16 st > C B - K - 15 on.
        const int zero_top = C * kB - num_taps - 15;
        const int st_cmax = zero_top < 0 ? 0 : zero_top / 16 + 1;
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        // Start-address fields (address / 16): chunk 0 of K-step st starts 16 C + 2 st strip
        // elements in and C blocks (2 C plane rows) into the stage; each next chunk is 16 strip
        // elements (128 units) and 2 rows (2 units) lower.
        const uint32_t a_hi0 = ((sbase + lay.taps_hi) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
        const uint32_t a_lo0 = ((sbase + lay.taps_lo) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
        const uint32_t b_base = ((sbase + lay.stages0) >> 4) + static_cast<uint32_t>(2 * C);
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        bool stop = false;
        int u = 0;   // K-steps issued (block-wide numbering)
        int g = 0;   // H groups issued
        for (int k = 0; k < my_tiles && !stop && !*abort; ++k) {
            if (!mbar_wait_bounded(smem_u32(&ctl.xempty[k & 1]), ((k >> 1) & 1) ^ 1, fault,
                                   kFaultAccumEmpty, abort)) {
                break;
            }
            fence_after();
            const uint32_t x_acc = tmem + kXCol + static_cast<uint32_t>(k & 1) * kN;
            for (int st0 = 0; st0 < kSteps && !stop; st0 += hks, ++g) {
                // (With one H group per tile, H and X of a tile are drained together and the
                // tile's X barriers guard both.)
                if (groups > 1 &&
                    !mbar_wait_bounded(smem_u32(&ctl.hempty[g & 1]), ((g >> 1) & 1) ^ 1, fault,
                                       kFaultAccumEmpty, abort)) {
                    stop = true;
                    break;
                }
                fence_after();
                const uint32_t h_acc = tmem + static_cast<uint32_t>(g & 1) * kN;
                const int st1 = min(kSteps, st0 + hks);
                for (int st = st0; st < st1; ++st, ++u) {
                    const int slot = u % stages;
                    if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (u / stages) & 1, fault,
                                           kFaultStageFull, abort)) {
                        stop = true;
                        break;
                    }
                    fence_after();
                    const uint32_t off = static_cast<uint32_t>(2 * st) * 8u;
                    unsigned long long dah = a_desc | (a_hi0 + off);
                    unsigned long long dal = a_desc | (a_lo0 + off);
                    unsigned long long dbh =
                        b_desc | (b_base + static_cast<uint32_t>(slot) * stage_units);
                    unsigned long long dbl = dbh + split_units;
                    const uint32_t h_first = st == st0 ? 0u : 1u;
                    const uint32_t x_first = st == 0 ? 0u : 1u;
                    const int c_end = st >= st_cmax ? C + 1 : C;
                    if (elect_one()) {
                        mma_f16<kIdesc>(h_acc, dah, dbh, h_first);
                        mma_f16<kIdesc>(x_acc, dah, dbl, x_first);
                        mma_f16_acc<kIdesc>(x_acc, dal, dbh);
                        for (int c = 1; c < c_end; ++c) {
                            dah -= 128;
                            dal -= 128;
                            dbh -= 2;
                            dbl -= 2;
                            mma_f16_acc<kIdesc>(h_acc, dah, dbh);
                            mma_f16_acc<kIdesc>(x_acc, dah, dbl);
                            mma_f16_acc<kIdesc>(x_acc, dal, dbh);
                        }
                        mma_commit(smem_u32(&ctl.empty[slot]));
                    }
                    __syncwarp();
                }
                if (groups > 1 && !stop && elect_one()) {
                    mma_commit(smem_u32(&ctl.hfull[g & 1]));
                }
                __syncwarp();
            }
            if (!stop && elect_one()) {
                mma_commit(smem_u32(&ctl.xfull[k & 1]));
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
        const uint32_t elem_off = static_cast<uint32_t>(q >> 2) * lay.pitch +
                                  static_cast<uint32_t>(q & 3) * 4u;
        // The thread's items are at the same places in every group: window offset (K-step g
        // of the group, row b, pair q) relative to the group's first K-step, and plane offset
        // relative to the group's first stage. The group's stages are consecutive slots (the
        // stage count is a multiple of kGroup). ~0 marks an unused item.
        uint32_t src_off[kItemIters];
        uint32_t dst_off[kItemIters];
#pragma unroll
        for (int i = 0; i < kItemIters; ++i) {
            const int f8 = (ptid >> 3) + (kProducers / 8) * i;   // g rows + b
            const int gi = f8 / rows;
            const int b = f8 - gi * rows;
            src_off[i] = f8 < kGroup * rows
                             ? static_cast<uint32_t>(b * 128 + 16 * gi + 2 * q) * (kPairBytes / 2)
                             : ~0u;
            dst_off[i] = static_cast<uint32_t>(gi) * lay.stage + elem_off +
                         static_cast<uint32_t>(2 * b) * 16u;
        }
        int u = 0;
        bool ok = true;
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            const int wb = k % wins;
            // The tile's scale (published by the scan warps once they scanned the window,
            // partial block included) and its window.
            if (!mbar_wait_bounded(smem_u32(&ctl.sready[k % kScales]), (k / kScales) & 1, fault,
                                   kFaultScale, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.win_full[wb]), (k / wins) & 1, fault,
                                   kFaultTileLoad, abort)) {
                break;
            }
            const uint32_t win = sbase + lay.win0 + static_cast<uint32_t>(wb) * lay.win;
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k % kScales]);
            const float fs = exp2_exact(ex);
            const f32x2 fs2 = pack2(fs, fs);
            for (int st0 = 0; st0 < kSteps && ok; st0 += kGroup, u += kGroup) {
#pragma unroll
                for (int gi = 0; gi < kGroup; ++gi) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.empty[(u + gi) % stages]),
                                           (((u + gi) / stages) & 1) ^ 1, fault,
                                           kFaultStageEmpty, abort)) {
                        ok = false;
                    }
                }
                if (!ok) {
                    break;
                }
                const uint32_t src0 = win + static_cast<uint32_t>(16 * st0) * (kPairBytes / 2);
                const uint32_t dst0 =
                    sbase + lay.stages0 + static_cast<uint32_t>(u % stages) * lay.stage;
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
                        sts32(row_re + lay.split, re_lo);
                        sts32(row_re + lay.split + 16u, im_lo);
                    }
                }
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) {
#pragma unroll
                    for (int gi = 0; gi < kGroup; ++gi) {
                        mbar_arrive(smem_u32(&ctl.full[(u + gi) % stages]));
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
        // ---- drain warps: H groups into running sums, then X, scaled, stored ----------------
        const int quarter = warp & 3;
        const int half = (warp - kFirstDrainWarp) >> 2;        // blocks kNB/2 half .. + kNB/2 - 1
        const int r = kB - 1 - (quarter * 32 + lane);          // output row of this TMEM lane
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(half * kNB);
        float acc[groups > 1 ? kNB : 1];
#pragma unroll
        for (int i = 0; i < (groups > 1 ? kNB : 1); ++i) {
            acc[i] = 0.0f;
        }
        // Adds this lane's kNB columns of the accumulator at column `col` into acc.
        auto add_columns = [&](uint32_t col) {
            if constexpr (groups > 1) {
#pragma unroll
                for (int c16 = 0; c16 < kNB / 16; ++c16) {
                    uint32_t t[16];
                    tmem_ld16(lane_addr + col + static_cast<uint32_t>(c16 * 16), t);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        acc[c16 * 16 + i] += __uint_as_float(t[i]);
                    }
                }
            }
        };
        bool ok = true;
        int g = 0;
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            if constexpr (groups == 1) {
                // One H group per tile: H and X read side by side, summed and stored per 16
                // columns (no running sums held across the tile).
                if (!mbar_wait_bounded(smem_u32(&ctl.xfull[k & 1]), (k >> 1) & 1, fault,
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
                const uint32_t hcol = static_cast<uint32_t>(g & 1) * kN;
                const uint32_t xcol = kXCol + static_cast<uint32_t>(k & 1) * kN;
#pragma unroll
                for (int c16 = 0; c16 < kNB / 16; ++c16) {
                    uint32_t th[16];
                    uint32_t tx[16];
                    tmem_ld16(lane_addr + hcol + static_cast<uint32_t>(c16 * 16), th);
                    tmem_ld16(lane_addr + xcol + static_cast<uint32_t>(c16 * 16), tx);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const long long o = (jb0 + c16 * 8 + i) * kB + r;
                        if (o < n) {
                            const float re =
                                __uint_as_float(th[2 * i]) + __uint_as_float(tx[2 * i]);
                            const float im =
                                __uint_as_float(th[2 * i + 1]) + __uint_as_float(tx[2 * i + 1]);
                            y[o] = make_float2(re * fa * fb, im * fa * fb);
                        }
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.xempty[k & 1]));
                }
                ++g;
                continue;
            }
            for (int gi = 0; gi < groups; ++gi, ++g) {
                if (!mbar_wait_bounded(smem_u32(&ctl.hfull[g & 1]), (g >> 1) & 1, fault,
                                       kFaultAccumFull, abort)) {
                    ok = false;
                    break;
                }
                fence_after();
                add_columns(static_cast<uint32_t>(g & 1) * kN);
                fence_before();
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.hempty[g & 1]));
                }
            }
            // The scale ring holds kScales tiles: tile k + 8's window lands only after the
            // producers converted tile k + 8 - wins, which needed the MMAs of that tile, which
            // needed tile k + 6 - wins (k + 3 at the most windows) drained: ex[k % kScales] is
            // read before it is rewritten.
            if (!ok ||
                !mbar_wait_bounded(smem_u32(&ctl.xfull[k & 1]), (k >> 1) & 1, fault,
                                   kFaultAccumFull, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.sready[k % kScales]), (k / kScales) & 1, fault,
                                   kFaultScale, abort)) {
                break;
            }
            fence_after();
            add_columns(kXCol + static_cast<uint32_t>(k & 1) * kN);
            fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.xempty[k & 1]));
            }
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k % kScales]);
            const int shift = -(ex + eh);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            const long long jb0 = tile_of(k) * kNB + half * (kNB / 2);
            if constexpr (groups > 1) {
#pragma unroll
                for (int i = 0; i < kNB / 2; ++i) {
                    const long long o = (jb0 + i) * kB + r;
                    if (o < n) {
                        y[o] = make_float2(acc[2 * i] * fa * fb, acc[2 * i + 1] * fa * fb);
                    }
                    acc[2 * i] = 0.0f;
                    acc[2 * i + 1] = 0.0f;
                }
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
            const int wb = j % wins;
            if (!mbar_wait_bounded(smem_u32(&ctl.win_full[wb]), (j / wins) & 1, fault,
                                   kFaultTileLoad, abort)) {
                break;
            }
            const uint32_t win = sbase + lay.win0 + static_cast<uint32_t>(wb) * lay.win;
            // The input's last, partial block lies outside the tensor map (its copy read
            // zeros): its stored samples go into their window row (only one tile of a block
            // holds that row), then the scan warps wait for each other.
            const long long rel = full_blocks - (tile_of(j) * kNB - C);
            if (tail > 0 && rel >= 0 && rel < rows) {   // uniform across the scan warps
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
                if (!mbar_wait_bounded(smem_u32(&ctl.patched), 0, fault, kFaultTileLoad, abort)) {
                    break;
                }
            }
            uint32_t m = 0;
            const int pairs = rows * 64;
#pragma unroll 4
            for (int f = stid; f < pairs; f += kScanWarps * 32) {
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

namespace {

constexpr uint32_t kSmemMax = 227u * 1024u;

}  // namespace

bool fir_tcw_supported(int num_taps)
{
    return num_taps >= 2 && (num_taps + kB - 2) / kB <= kCMax &&
           win_layout(num_taps, kWins, kStages, 4).bytes <= kSmemMax;
}

long long fir_tcw_tile_outputs() { return static_cast<long long>(kNB) * kB; }

template <int C, int kFmt>
static cudaError_t launch_tcw(const void* x, const float* taps, void* y, long long n, int num_taps,
                              cudaStream_t stream)
{
    constexpr int es = component_bytes(kFmt);
    const Layout lay = win_layout(num_taps, kWins, kStages, es);
    if (lay.bytes > kSmemMax) {
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
    err = encode_rows(&map, x, es, n / kB, 2 * kB, 2 * kB, static_cast<uint32_t>(lay.rows));
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + kB - 1) / kB;
    const int tiles = static_cast<int>((blocks + kNB - 1) / kNB);
    const int grid = tiles < sms ? tiles : sms;
    fir_tcw_kernel<C, kFmt><<<grid, kThreads, bytes, stream>>>(
        map, x, taps, static_cast<float2*>(y), n, num_taps, tiles);
    return cudaGetLastError();
}

cudaError_t fir_tcw_launch(int format, const void* x, const float* taps, void* y, long long n,
                           int num_taps, cudaStream_t stream)
{
    if (n < kB || !fir_tcw_supported(num_taps)) {
        return cudaErrorInvalidValue;
    }
    const int C = (num_taps + kB - 2) / kB;
    if (format < 0 || format > 2) {
        return cudaErrorInvalidValue;
    }
    static cudaError_t (*const launchers[kCMax][3])(const void*, const float*, void*, long long,
                                                     int, cudaStream_t) = {
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
