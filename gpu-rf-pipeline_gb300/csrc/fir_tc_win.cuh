// The resident-window tensor-core FIR pipeline (2 to 385 taps) as a device-side template, run by
// the single-capture kernel (fir_tc_win.cu) and by the batch kernel's window phase
// (fir_batch.cu). The algorithm, its roles and their measured costs are described in
// fir_tc_win.cu; this header holds the pipeline and the two ways it finds its tiles:
//  * TcwSingleSrc: one capture, tile k of a block = blockIdx.x + k gridDim.x;
//  * TcwListSrc: a contiguous range of (capture, tile) work items, captures in increasing order,
//    each with its own taps, length and tensor map (in global memory). The tap strip is then
//    rebuilt per capture by the scan warps, into one of two strip slots or into the only one
//    (kStrips), after the MMA warp's `strip_free` commit for the capture that used the slot
//    last, and published with `strip_ready`; the scan warps publish the capture's first tile
//    scale before they wait for the slot, and the drain's tap scale travels with each tile's
//    sample scale.
#pragma once

#include "sample_fmt.cuh"
#include "tc_common.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {
namespace tcw {

using namespace tc;

constexpr int kB = 128;                   // outputs per block = MMA M
constexpr int kNB = 48;                   // blocks per tile; MMA N = 2 * kNB
constexpr int kN = 2 * kNB;
constexpr int kCMax = 3;                  // blocks a block reaches back to, at most (385 taps)
constexpr int kRowsMax = kNB + kCMax;     // window rows per tile, at most
constexpr int kSteps = kB / 16;           // K-steps of 16 samples per tile
constexpr int kWins = 3;                  // window buffers
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
constexpr uint32_t kSmemMax = 227u * 1024u;
static_assert(kNB % 16 == 0, "a drain warp reads its kNB columns 16 at a time");

// One capture as the pipeline sees it.
struct WinCapture {
    const void* x;        // samples as stored (cf32, ci16 or ci8)
    float2* y;
    const float* taps;
    long long n;
    int num_taps;
    int item0;            // first work item of this capture (a list of captures)
};

// Shared-memory layout (window buffers, stages, strip slots and the sample format fixed).
struct Layout {
    int tcount;          // core matrices of a tap strip: 16 C + 31
    uint32_t pitch;      // bytes per plane: 2 rows x 16 B per block + 16 (banks)
    uint32_t split;      // one split (hi or lo) of a stage: 2 planes
    uint32_t stage;      // one operand stage: hi + lo
    uint32_t win;        // one window buffer: rows x 256 components
    uint32_t taps0;      // first strip slot (hi, then lo); the next slot follows
    uint32_t strip;      // bytes of one strip slot (hi + lo)
    uint32_t stages0, win0, bytes;
};

__host__ __device__ inline Layout win_layout(int C, int stages, int strips, int es)
{
    Layout l;
    const int rows = kNB + C;
    l.tcount = 16 * C + 31;
    l.pitch = static_cast<uint32_t>(2 * rows) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    l.win = static_cast<uint32_t>(rows) * 256u * static_cast<uint32_t>(es);
    l.taps0 = 1024;
    l.strip = 2u * 128u * static_cast<uint32_t>(l.tcount);
    l.stages0 = (l.taps0 + static_cast<uint32_t>(strips) * l.strip + 1023u) & ~1023u;
    l.win0 = (l.stages0 + static_cast<uint32_t>(stages) * l.stage + 1023u) & ~1023u;
    l.bytes = l.win0 + static_cast<uint32_t>(kWins) * l.win;
    return l;
}

struct Ctrl {
    unsigned long long full[8];          // stage converted (every producer warp)
    unsigned long long empty[8];         // stage read by its MMAs (tcgen05.commit)
    unsigned long long win_full[kWins];  // window copied (transaction bytes)
    unsigned long long win_empty[kWins]; // window converted (every producer warp)
    unsigned long long hfull[2];         // an H group summed (tcgen05.commit)
    unsigned long long hempty[2];        // an H group read (every drain warp)
    unsigned long long xfull[2];         // a tile's X summed (tcgen05.commit)
    unsigned long long xempty[2];        // a tile's X read (every drain warp)
    unsigned long long sready[kScales];  // the scales of tile k are in ex/ehr[k % kScales]
    unsigned long long pready[2];        // every scan warp's part of a window's maximum written
    unsigned long long patched;          // the partial last block written into its window row
    unsigned long long strip_ready[2];   // a strip slot built (every scan warp)
    unsigned long long strip_free[2];    // the MMAs reading a strip slot done (tcgen05.commit)
    unsigned long long teardown;
    int abort;
    uint32_t pmax[2][kScanWarps];
    int ex[kScales];                     // sample scale exponent of a tile
    int ehr[kScales];                    // tap scale exponent of a tile's capture
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// Makes a tensor map that the host wrote into global memory visible to the tensor-map proxy
// of the calling thread before its first TMA copy through it.
__device__ __forceinline__ void tmap_acquire_global(const CUtensorMap* map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// A role's place in the capture list: the capture index and the items it holds, in registers,
// so that a lookup reads the list only when an item passes into the next capture.
struct TcwCursor {
    int idx = -1;
    int item0 = 0;
    int end = 0;   // first item of the next capture
};

struct TcwSingleSrc {
    static constexpr bool kMulti = false;
    const CUtensorMap* map;   // in the kernel parameters
    WinCapture cap;
    int tiles;
    __device__ int count() const
    {
        return static_cast<int>(blockIdx.x) < tiles
                   ? (tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                   : 0;
    }
    __device__ void locate(int k, TcwCursor& cur, long long& t) const
    {
        cur.idx = 0;
        cur.end = 0x7fffffff;
        t = static_cast<long long>(blockIdx.x) + static_cast<long long>(k) * gridDim.x;
    }
    __device__ const WinCapture& capture(int) const { return cap; }
    __device__ const CUtensorMap* tmap(int) const { return map; }
    __device__ void acquire(int, int&) const {}
};

struct TcwListSrc {
    static constexpr bool kMulti = true;
    const WinCapture* caps;   // in global memory, item0 increasing
    const CUtensorMap* maps;  // in global memory, one per capture
    int ncaps;
    int first;                // this block's items: first .. first + items - 1
    int items;
    __device__ int count() const { return items; }
    // Capture and tile of the block's k-th item: the cursor moves forward only when the item
    // leaves its capture (its first position by binary search: a forward scan from the list's
    // start cost every role of a late block a chain of dependent loads per phase).
    __device__ void locate(int k, TcwCursor& cur, long long& t) const
    {
        const int item = first + k;
        if (item >= cur.end) {
            int i = cur.idx + 1;
            if (cur.idx < 0) {
                int hi = ncaps - 1;
                i = 0;
                while (i < hi) {
                    const int mid = (i + hi + 1) >> 1;
                    if (caps[mid].item0 <= item) {
                        i = mid;
                    } else {
                        hi = mid - 1;
                    }
                }
            } else {
                while (i + 1 < ncaps && caps[i + 1].item0 <= item) {
                    ++i;
                }
            }
            cur.idx = i;
            cur.item0 = caps[i].item0;
            cur.end = i + 1 < ncaps ? caps[i + 1].item0 : 0x7fffffff;
        }
        t = item - cur.item0;
    }
    __device__ const WinCapture& capture(int c) const { return caps[c]; }
    __device__ const CUtensorMap* tmap(int c) const { return maps + c; }
    // Fences the maps up to capture c, from the thread's first capture on (the only ones it
    // copies through).
    __device__ void acquire(int c, int& fenced) const
    {
        if (fenced < 0) {
            fenced = c - 1;
        }
        for (; fenced < c; ++fenced) {
            tmap_acquire_global(maps + fenced + 1);
        }
    }
};

// The tap strip G[t][q][e] = 2^eh h[(C + 1) B - 1 - 8 t - q - e], FP16 hi and lo, built by the
// `nthreads` threads numbered `tid` (two adjacent elements e, e + 1 of core matrix t, row q per
// item).
template <int C>
__device__ __forceinline__ void build_strip(uint32_t hi, uint32_t lo, const float* taps,
                                            int num_taps, int eh, int tid, int nthreads)
{
    const float fa = exp2i(eh / 2);
    const float fb = exp2i(eh - eh / 2);
    constexpr int dmax = (C + 1) * kB - 1;
    for (int i = tid; i < (16 * C + 31) * 32; i += nthreads) {
        const int t = i >> 5;
        const int q = (i >> 2) & 7;
        const int e = (i & 3) * 2;
        const int i0 = dmax - 8 * t - q - e;
        const int i1 = i0 - 1;
        const float v0 = (i0 >= 0 && i0 < num_taps) ? __ldg(taps + i0) * fa * fb : 0.0f;
        const float v1 = (i1 >= 0 && i1 < num_taps) ? __ldg(taps + i1) * fa * fb : 0.0f;
        uint32_t h, l;
        split2(v0, v1, h, l);
        const uint32_t off = static_cast<uint32_t>(t) * 128u + q * 16u + e * 2u;
        sts32(hi + off, h);
        sts32(lo + off, l);
    }
}

// The pipeline over the block's tiles of `src`. `smem` is the dynamic shared memory (the layout
// from offset 1024), `ctl` its control block (anywhere outside the layout), `tmem` 512 columns
// this block owns, `fault` the fault word. Every thread of the block calls it (kThreads of them:
// warps beyond the roles return at the final barrier) and returns after a block barrier.
// With a list of captures (kMulti) the caller invalidates the control block's barriers before
// the memory is used for anything else (tcw_release).
template <int C, int kFmt, int S, class Src, int kStrips = 2>
__device__ __forceinline__ void tcw_pipeline(const Src& src, unsigned char* smem, Ctrl& ctl,
                                             uint32_t tmem, unsigned int* fault)
{
    constexpr bool kMulti = Src::kMulti;
    constexpr int es = component_bytes(kFmt);
    constexpr uint32_t kPairBytes = 4u * es;   // two samples as stored
    constexpr int rows = kNB + C;
    constexpr int hks = kSteps < kHGroup / (C + 1) ? kSteps : kHGroup / (C + 1);
    constexpr int groups = (kSteps + hks - 1) / hks;
    constexpr int wins = kWins;
    constexpr int stages = S;
    constexpr int kGroup = S / 2;             // K-steps the producers convert at once
    // A group's items (K-step g, row b, sample pair q), numbered f = (g rows + b) 8 + q, are
    // dealt to the producer threads in turn: thread t takes f = t, t + kProducers, ... (q = t % 8
    // throughout, so eight consecutive lanes write one 16-byte plane row each: no bank
    // conflicts).
    constexpr int kItemIters = (kGroup * rows * 8 + kProducers - 1) / kProducers;
    static_assert(hks >= 1, "an H group holds at least one K-step");
    static_assert(S == 4 || S == 8, "4 or 8 operand stages");
    static_assert(kSteps % kGroup == 0, "producer groups");
    const Layout lay = win_layout(C, stages, kMulti ? kStrips : 1, es);
    // The warp index through a shuffle: provably the same on every lane of a warp, so values
    // derived from it in a role's loop can stay in uniform registers.
    const int warp = __shfl_sync(0xFFFFFFFFu, static_cast<int>(threadIdx.x >> 5), 0);
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    const int my_tiles = src.count();
    TcwCursor copy_cursor;   // the copy thread's capture cursor and the maps it has fenced
    int fenced = -1;
    auto issue_window = [&](int k) {
        long long t;
        src.locate(k, copy_cursor, t);
        src.acquire(copy_cursor.idx, fenced);
        const uint32_t bar = smem_u32(&ctl.win_full[k % wins]);
        mbar_arrive_expect_tx(bar, lay.win);
        tma_load_2d(sbase + lay.win0 + static_cast<uint32_t>(k % wins) * lay.win,
                    src.tmap(copy_cursor.idx), 0, static_cast<int>(t * kNB - C), bar);
    };
    auto strip_hi = [&](int slot) {
        return sbase + lay.taps0 + static_cast<uint32_t>(slot) * lay.strip;
    };
    auto strip_lo = [&](int slot) { return strip_hi(slot) + lay.strip / 2u; };
    // With a list of captures, capture number occ (of those this block meets) builds its strip
    // in slot strip_slot(occ), after strip_use(occ) earlier captures used that slot.
    static_assert(kStrips == 1 || kStrips == 2, "one or two tap-strip slots");
    auto strip_slot = [](int occ) { return kStrips == 2 ? (occ & 1) : 0; };
    auto strip_use = [](int occ) { return kStrips == 2 ? (occ >> 1) : occ; };

    // ---- setup: barriers, the first windows, the tap strip of a single capture -------------
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
            mbar_init(smem_u32(&ctl.strip_ready[i]), kScanWarps);
            mbar_init(smem_u32(&ctl.strip_free[i]), 1);
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
    int eh_single = 0;         // the tap scale of a single capture
    if constexpr (!kMulti) {
        const WinCapture& cap = src.capture(0);
        uint32_t m = 0;
        for (int k = threadIdx.x; k < cap.num_taps; k += kThreads) {
            m = max(m, absbits(__ldg(cap.taps + k)));
        }
        m = __reduce_max_sync(0xFFFFFFFFu, m);
        __syncthreads();   // tap_max initialised
        if (lane == 0 && m != 0) {
            atomicMax(&ctl.tap_max, m);
        }
        __syncthreads();
        eh_single = scale_exponent(ctl.tap_max);
        build_strip<C>(strip_hi(0), strip_lo(0), cap.taps, cap.num_taps, eh_single,
                       threadIdx.x, kThreads);
    }
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
    fence_after();

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
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        // Start-address fields (address / 16): chunk 0 of K-step st starts 16 C + 2 st strip
        // elements in and C blocks (2 C plane rows) into the stage; each next chunk is 16 strip
        // elements (128 units) and 2 rows (2 units) lower.
        const uint32_t b_base = ((sbase + lay.stages0) >> 4) + static_cast<uint32_t>(2 * C);
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        bool stop = false;
        int u = 0;     // K-steps issued (block-wide numbering)
        int g = 0;     // H groups issued
        TcwCursor cur;
        int occ = -1;  // captures met so far
        int cap_now = -1;
        int st_cmax = 0;
        uint32_t a_hi0 = 0;
        uint32_t a_lo0 = 0;
        for (int k = 0; k < my_tiles && !stop && !*abort; ++k) {
            long long t;
            src.locate(k, cur, t);
            if (cur.idx != cap_now) {
                // A new capture: its strip slot, and the first K-step whose last chunk holds
                // taps (16 st > C B - K - 15).
                cap_now = cur.idx;
                ++occ;
                if constexpr (kMulti) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.strip_ready[strip_slot(occ)]),
                                           strip_use(occ) & 1,
                                           fault, kFaultStageFull, abort)) {
                        break;
                    }
                }
                const int zero_top = C * kB - src.capture(cur.idx).num_taps - 15;
                st_cmax = zero_top < 0 ? 0 : zero_top / 16 + 1;
                a_hi0 = (strip_hi(strip_slot(occ)) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
                a_lo0 = (strip_lo(strip_slot(occ)) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
            }
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
            if constexpr (kMulti) {
                // The capture's last tile of this block: its strip slot is free once these
                // MMAs complete.
                TcwCursor next = cur;
                long long tn;
                if (k + 1 < my_tiles) {
                    src.locate(k + 1, next, tn);
                }
                if (!stop && (k + 1 == my_tiles || next.idx != cur.idx) && elect_one()) {
                    mma_commit(smem_u32(&ctl.strip_free[strip_slot(occ)]));
                }
                __syncwarp();
            }
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
                    uint32_t tt[16];
                    tmem_ld16(lane_addr + col + static_cast<uint32_t>(c16 * 16), tt);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        acc[c16 * 16 + i] += __uint_as_float(tt[i]);
                    }
                }
            }
        };
        bool ok = true;
        int g = 0;
        TcwCursor cur;
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            long long t;
            src.locate(k, cur, t);
            // The capture's output and length in registers for the tile's stores.
            float2* const cap_y = src.capture(cur.idx).y;
            const long long cap_n = src.capture(cur.idx).n;
            const long long jb0 = t * kNB + half * (kNB / 2);
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
                const int eh = *reinterpret_cast<volatile int*>(&ctl.ehr[k % kScales]);
                const int shift = -(ex + eh);
                const float fa = exp2i(shift / 2);
                const float fb = exp2i(shift - shift / 2);
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
                        if (o < cap_n) {
                            const float re =
                                __uint_as_float(th[2 * i]) + __uint_as_float(tx[2 * i]);
                            const float im =
                                __uint_as_float(th[2 * i + 1]) + __uint_as_float(tx[2 * i + 1]);
                            cap_y[o] = make_float2(re * fa * fb, im * fa * fb);
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
            // needed tile k + 6 - wins (k + 3) drained: the entries of tile k are read before
            // they are rewritten.
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
            const int eh = *reinterpret_cast<volatile int*>(&ctl.ehr[k % kScales]);
            const int shift = -(ex + eh);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            if constexpr (groups > 1) {
#pragma unroll
                for (int i = 0; i < kNB / 2; ++i) {
                    const long long o = (jb0 + i) * kB + r;
                    if (o < cap_n) {
                        cap_y[o] = make_float2(acc[2 * i] * fa * fb, acc[2 * i + 1] * fa * fb);
                    }
                    acc[2 * i] = 0.0f;
                    acc[2 * i + 1] = 0.0f;
                }
            }
        }
    } else if (warp < kFirstScanWarp + kScanWarps) {
        // ---- scan warps: each capture's tap strip, each window's scale as soon as it lands --
        // The largest |component| of the window brought into [2^14, 2^15), clamped to 127 so
        // that 2^ex is one float and the scaling one exact multiply, published to the producers
        // and the drain warps with the capture's tap scale. A separate role, so that a scale
        // never waits behind a drain.
        const int sw = warp - kFirstScanWarp;
        const int stid = static_cast<int>(threadIdx.x) - kFirstScanWarp * 32;
        TcwCursor cur;
        int occ = -1;
        int cap_now = -1;
        int patches = 0;   // partial blocks written (phases of `patched`)
        int eh = eh_single;
        for (int j = 0; j < my_tiles && !*abort; ++j) {
            long long t;
            src.locate(j, cur, t);
            const WinCapture& cap = src.capture(cur.idx);
            const bool new_cap = cur.idx != cap_now;
            if (new_cap) {
                cap_now = cur.idx;
                ++occ;
                if constexpr (kMulti) {
                    // The capture's tap scale (each scan warp takes the whole maximum); its
                    // strip follows the scale of its first tile, below.
                    uint32_t m = 0;
                    for (int i = lane; i < cap.num_taps; i += 32) {
                        m = max(m, absbits(__ldg(cap.taps + i)));
                    }
                    eh = scale_exponent(__reduce_max_sync(0xFFFFFFFFu, m));
                }
            }
            const int wb = j % wins;
            if (!mbar_wait_bounded(smem_u32(&ctl.win_full[wb]), (j / wins) & 1, fault,
                                   kFaultTileLoad, abort)) {
                break;
            }
            const uint32_t win = sbase + lay.win0 + static_cast<uint32_t>(wb) * lay.win;
            // The capture's last, partial block lies outside its tensor map (the copy read
            // zeros): its stored samples go into their window row (only one tile of a capture
            // holds that row), then the scan warps wait for each other. With a list of
            // captures this happens once per capture: the barrier's phase counts them.
            const long long full_blocks = cap.n / kB;
            const int tail = static_cast<int>(cap.n - full_blocks * kB);
            const long long rel = full_blocks - (t * kNB - C);
            if (tail > 0 && rel >= 0 && rel < rows) {   // uniform across the scan warps
                const uint32_t row = win + static_cast<uint32_t>(rel) * 256u * es;
                for (int i = stid; i < tail; i += kScanWarps * 32) {
                    const long long sidx = full_blocks * kB + i;
                    if constexpr (kFmt == 0) {
                        const float2 v = __ldg(static_cast<const float2*>(cap.x) + sidx);
                        sts64(row + static_cast<uint32_t>(i) * 8u, pack2(v.x, v.y));
                    } else if constexpr (kFmt == 1) {
                        sts32(row + static_cast<uint32_t>(i) * 4u,
                              __ldg(static_cast<const unsigned int*>(cap.x) + sidx));
                    } else {
                        const unsigned short v =
                            __ldg(static_cast<const unsigned short*>(cap.x) + sidx);
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
                if (!mbar_wait_bounded(smem_u32(&ctl.patched), patches & 1, fault, kFaultTileLoad,
                                       abort)) {
                    break;
                }
                ++patches;
            }
            uint32_t m = 0;
            constexpr int pairs = rows * 64;
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
                ctl.ehr[j % kScales] = eh;
                mbar_arrive(smem_u32(&ctl.sready[j % kScales]));
            }
            if constexpr (kMulti) {
                if (new_cap) {
                    // The capture's strip, into its slot once the MMAs of the capture that used
                    // the slot last are done; after the first tile's scale, so that the
                    // producers convert that tile meanwhile. Each scan warp builds half.
                    const int slot = strip_slot(occ);
                    if (!mbar_wait_bounded(smem_u32(&ctl.strip_free[slot]),
                                           (strip_use(occ) & 1) ^ 1, fault, kFaultStageEmpty,
                                           abort)) {
                        break;
                    }
                    build_strip<C>(strip_hi(slot), strip_lo(slot), cap.taps, cap.num_taps, eh,
                                   stid, kScanWarps * 32);
                    fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) {
                        mbar_arrive(smem_u32(&ctl.strip_ready[slot]));
                    }
                }
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
}

// Invalidates the control block's barriers of a pipeline run with S stages (one thread, after
// the pipeline returned), so that their memory can serve another purpose.
template <int S>
__device__ __forceinline__ void tcw_release(Ctrl& ctl)
{
    auto inval = [](unsigned long long* b) {
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(b)) : "memory");
    };
    for (int i = 0; i < S; ++i) {
        inval(&ctl.full[i]);
        inval(&ctl.empty[i]);
    }
    for (int i = 0; i < kWins; ++i) {
        inval(&ctl.win_full[i]);
        inval(&ctl.win_empty[i]);
    }
    for (int i = 0; i < 2; ++i) {
        inval(&ctl.hfull[i]);
        inval(&ctl.hempty[i]);
        inval(&ctl.xfull[i]);
        inval(&ctl.xempty[i]);
        inval(&ctl.pready[i]);
        inval(&ctl.strip_ready[i]);
        inval(&ctl.strip_free[i]);
    }
    for (int i = 0; i < kScales; ++i) {
        inval(&ctl.sready[i]);
    }
    inval(&ctl.patched);
    inval(&ctl.teardown);
}

}  // namespace tcw
}  // namespace rfx
