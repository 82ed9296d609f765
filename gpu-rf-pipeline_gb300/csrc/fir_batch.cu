// Batched tensor-core FIR: many captures, each with its own taps and length, in ONE persistent
// launch. No counterpart in the project, which runs such a batch as one launch per capture.
//
// Work list: every capture is cut into tiles of 96 blocks of 128 outputs (as fir_tc.cu); the
// (capture, tile) items are numbered capture by capture, and each block of the grid takes one
// contiguous range of items, the ranges chosen on the host so that every block gets about the
// same work (measured: about the same per tile whatever the filter). The capture table,
// including each capture's two TMA tensor maps, travels in the kernel parameters (304 bytes per
// capture, 96 captures per launch), so a launch allocates nothing and can be captured in a CUDA
// graph.
//
// The per-tile pipeline is the one of fir_tc.cu, roles included: 16 drain warps hold the FP32
// running sums and write the outputs; 7 producer warps compute each tile's scale from TMA scan
// slices of its window, convert each K-step's samples (arriving by 2-D TMA copies, zero fill
// outside the capture) into scaled FP16 hi/lo planes, and keep the copies flowing; one thread
// issues the MMAs (h_hi x_hi into accumulator H in groups of at most 18, the cross products
// into X once per tile). What the batch adds:
//  * every quantity of a tile (window rows, tensor maps, partial last block, outputs) comes from
//    its capture;
//  * the shared-memory buffers are sized for the largest filter of the launch; the operand
//    planes keep that pitch for every capture, so the sample descriptors do not change;
//  * when a block's range moves on to the next capture, the producers rebuild the tap strip —
//    after the MMA thread has committed the last MMA of the previous capture (`strip_free`),
//    before the first stage of the new capture is marked full;
//  * the drain's scale is per tile: 2^-(ex + eh), eh the tile's capture's tap scale.
//
// A batch plan (work list in device memory) runs, in the same launch and after those items, the
// resident-window pipeline of fir_tc_win.cuh over its captures of 2 to 385 taps: one phase per
// reach-back C = 1, 2, 3 (the window geometry is compile-time), each block taking a contiguous
// range of that phase's 48-block tiles; the scan warps rebuild the tap strip at every capture
// switch into one of two slots, the MMA warp freeing a slot after its capture's last tile. Last
// come the plain tiles of the captures below 2 taps (the plain kernel's tile function:
// bit-exact). Tensor memory is allocated once per block for every phase.
#include "fir_tc.cuh"
#include "fir_plain.cuh"
#include "fir_plain_tile.cuh"
#include "tc_common.cuh"
#include "tmap.hpp"
#include "tuning.hpp"
#include "fir_tc_win.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace rfx {

static __device__ unsigned int g_fault_fir_batch;

namespace {

using namespace tc;

constexpr int kB = 128;
constexpr int kNB = 96;
constexpr int kN = 2 * kNB;
constexpr int kStagesPerTile = kB / 16;
constexpr int kDrainWarps = 16;
constexpr int kProducerWarps = 7;
constexpr int kProducers = kProducerWarps * 32;
constexpr int kFirstProducerWarp = kDrainWarps;
constexpr int kMmaWarp = kDrainWarps + kProducerWarps;
constexpr int kThreads = (kMmaWarp + 1) * 32;
constexpr int kCols = kN / 4;
constexpr int kHGroup = 18;       // MMAs per H accumulation, at most
constexpr int kRaw = 3;           // TMA raw-sample ring depth
constexpr int kScanBufsMax = 4;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kXCol = kN;
constexpr uint32_t kIdesc = idesc_f16(kB, kN);
constexpr int kBatchCaps = 96;    // captures per launch (the parameter space holds their maps)
constexpr int kBatchCtas = 160;   // blocks per launch at most (one per SM)

struct BatchCap {
    const float2* x;
    float2* y;
    const float* taps;
    long long n;
    int num_taps;
    int C;                // previous blocks a block reaches back to
    int tiles;
    int item0;            // first item of this capture in the work list
};

struct BatchParams {
    CUtensorMap xmap[kBatchCaps];  // x as rows of 256 floats (full blocks), boxes 32 x rows
    CUtensorMap smap[kBatchCaps];  // the same rows, boxes 256 floats x srows (scan slices)
    BatchCap cap[kBatchCaps];
    int count;
    int cmax;
    int sbufs;
    int cta_item[kBatchCtas + 1];
};
static_assert(sizeof(BatchParams) <= 32000, "kernel parameter space");

// A capture the batch runs on the plain kernel's tile function: its tiles of 2304 outputs are
// plain tiles tile0 .. tile0 + ceil(n / 2304) - 1 of the launch.
struct PlainCapDev {
    const float2* x;
    float2* y;
    const float* taps;
    long long n;
    int num_taps;
    int tile0;
};

// Where a launch finds its work: the tensor-core captures (table, tensor maps, item ranges per
// block) and the plain captures (table, plain-tile ranges per block). For rfx_fir_batch_launch
// the arrays are in the kernel parameters (BatchParams; no plain captures); for a batch plan
// they are in device memory, written once when the plan is made.
struct BatchView {
    const BatchCap* cap;
    const CUtensorMap* xmap;
    const CUtensorMap* smap;
    const int* cta_item;
    const PlainCapDev* pcap;
    const int* cta_plain;
    int count;
    int pcount;
    int cmax;
    int sbufs;
    int plain_groups;        // groups of 256 threads running plain tiles (0: none)
    uint32_t plain_region;   // shared-memory bytes per group
    uint32_t plain_slot;     // bytes per tile slot: region = 2 slots (pipelined) or 1
    int maps_global;         // tensor maps in global memory: fence them before first use
    // Captures for the resident-window pipeline (fir_tc_win.cuh), by blocks reached back C =
    // 1, 2, 3: capture list, window tensor maps, per-block item ranges; its control block sits
    // in the last kilobyte of shared memory (win_ctl), clear of every other phase's barriers.
    const tcw::WinCapture* wcap[tcw::kCMax];
    const CUtensorMap* wmap[tcw::kCMax];
    const int* cta_win[tcw::kCMax];
    int wcount[tcw::kCMax];
    uint32_t win_ctl;
};

// Per-capture window geometry.
struct Geo {
    int C;
    int rows;              // window blocks per tile: kNB + C
    int srows;             // window rows per scan slice
    uint32_t raw_tx;       // bytes of one raw copy: rows * 32 floats
    uint32_t scan_tx;      // bytes of one scan copy: srows * 256 floats
    long long full_blocks; // rows the tensor maps cover
};

__host__ __device__ inline Geo geo_of(int C, long long n)
{
    Geo g;
    g.C = C;
    g.rows = kNB + C;
    g.srows = (g.rows + kStagesPerTile - 1) / kStagesPerTile;
    g.raw_tx = static_cast<uint32_t>(g.rows) * 128u;
    g.scan_tx = static_cast<uint32_t>(g.srows) * 1024u;
    g.full_blocks = n / kB;
    return g;
}

// Shared memory, sized for the largest filter of the launch (cmax).
struct Layout {
    uint32_t pitch;       // bytes per plane: 2 rows * 16 B per window block (+16)
    uint32_t split;
    uint32_t stage;
    uint32_t raw;         // raw stage pitch
    uint32_t scan;        // scan slice pitch
    int tcount;           // core matrices of the largest tap strip
    uint32_t taps_hi, taps_lo, raw0, scan0, stages0, bytes;
};

__host__ __device__ inline Layout batch_layout(int cmax, int stages, int sbufs)
{
    const Geo g = geo_of(cmax, 0);
    Layout l;
    l.pitch = static_cast<uint32_t>(2 * g.rows) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    l.raw = (g.raw_tx + 127u) & ~127u;
    l.scan = (g.scan_tx + 127u) & ~127u;
    l.tcount = 16 * cmax + 31;
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount);
    l.raw0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount) + 127u) & ~127u;
    l.scan0 = l.raw0 + kRaw * l.raw;
    l.stages0 = l.scan0 + static_cast<uint32_t>(sbufs) * l.scan;
    l.bytes = l.stages0 + l.stage * static_cast<uint32_t>(stages);
    return l;
}

struct Ctrl {
    unsigned long long full[8];
    unsigned long long empty[8];
    unsigned long long raw_full[kRaw];
    unsigned long long raw_empty[kRaw];
    unsigned long long scan_full[kScanBufsMax];
    unsigned long long scan_empty[kScanBufsMax];
    unsigned long long pfull;
    unsigned long long pempty;
    unsigned long long xfull;
    unsigned long long xempty;
    unsigned long long sready[4];   // the output scale of item k is in shift[k % 4]
    unsigned long long strip_free;  // every MMA of the previous capture has completed
    unsigned long long teardown;
    int abort;
    uint32_t pmax[2][kProducerWarps];
    uint32_t tmaxw[2][kProducerWarps];
    // Item k's output description for the drain warps (slot k % 4, published with sready):
    // its capture's output and length, its first output block, its H groups, ex + eh.
    float2* item_y[4];
    long long item_n[4];
    long long item_block0[4];
    int item_groups[4];
    int shift[4];
};
static_assert(sizeof(Ctrl) <= 1020, "control block (the last word carries the TMEM base)");

// The capture holding work-list item `item` (binary search over the captures' first items).
__device__ __forceinline__ int capture_find(const BatchView& p, int item)
{
    int lo = 0;
    int hi = p.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.cap[mid].item0 <= item) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    return lo;
}

// A role's copy, in registers, of the fields of the capture that holds its current item,
// reloaded only when the item passes into the next capture (items only increase). Looking the
// capture up in the table on every K-step kept the producers' critical path waiting on loads:
// measured 145 against 124 us at 511 taps, 2^24 samples.
struct CapCursor {
    int idx;      // capture index
    int end;      // first item of the next capture
    int item0;    // first item of this capture
    int C;
    long long n;
};

__device__ __forceinline__ void cursor_load(const BatchView& p, int i, CapCursor& r)
{
    const BatchCap& c = p.cap[i];
    r.idx = i;
    r.item0 = c.item0;
    r.C = c.C;
    r.n = c.n;
    r.end = i + 1 < p.count ? p.cap[i + 1].item0 : 0x7fffffff;
}

// Moves the cursor on to the capture of `item`; true if it moved.
__device__ __forceinline__ bool cursor_seek(const BatchView& p, int item, CapCursor& r)
{
    bool moved = false;
    while (item >= r.end) {
        cursor_load(p, r.idx + 1, r);
        moved = true;
    }
    return moved;
}

// H groups of a tile with P chunks (see fir_tc.cu).
struct HGroups {
    int ksg;
    int gpk;
    int cpg;
    int per_tile;
};

__host__ __device__ inline HGroups h_groups(int P, int S)
{
    HGroups g;
    if (P <= kHGroup) {
        g.ksg = max(1, min(kHGroup / P, S - 1));
        g.gpk = 1;
        g.cpg = P;
        g.per_tile = (kStagesPerTile + g.ksg - 1) / g.ksg;
    } else {
        g.ksg = 1;
        g.gpk = (P + kHGroup - 1) / kHGroup;
        g.cpg = (P + g.gpk - 1) / g.gpk;
        g.gpk = (P + g.cpg - 1) / g.cpg;
        g.per_tile = kStagesPerTile * g.gpk;
    }
    return g;
}

__device__ __forceinline__ void h_group_range(const HGroups& g, int P, int gi, int& st0, int& st1,
                                              int& c0, int& c1)
{
    if (g.gpk == 1) {
        st0 = gi * g.ksg;
        st1 = min(kStagesPerTile, st0 + g.ksg);
        c0 = 0;
        c1 = P;
    } else {
        st0 = gi / g.gpk;
        st1 = st0 + 1;
        c0 = (gi - st0 * g.gpk) * g.cpg;
        c1 = min(P, c0 + g.cpg);
    }
}

}  // namespace

// Makes a tensor map that the host wrote into global memory visible to the tensor-map proxy
// of the calling thread before its first TMA copy through it.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap* map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// The tensor-core items first_item .. first_item + my_items - 1 of the work list (my_items > 0,
// the same for every thread of the block). Every thread returns after a final block barrier.
template <int S>
__device__ __forceinline__ void batch_tc_items(const BatchView& p, int first_item, int my_items,
                                               unsigned char* smem, uint32_t tmem)
{
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const int sbufs = p.sbufs;
    const Layout lay = batch_layout(p.cmax, S, sbufs);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_batch;
    const int my_steps = my_items * kStagesPerTile;
    const int scan_slices = (my_items - 1) * kStagesPerTile;
    const int cap_first = capture_find(p, first_item);

    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < kRaw; ++i) {
            mbar_init(smem_u32(&ctl.raw_full[i]), 1);
            mbar_init(smem_u32(&ctl.raw_empty[i]), kProducerWarps);
        }
        for (int i = 0; i < sbufs; ++i) {
            mbar_init(smem_u32(&ctl.scan_full[i]), 1);
            mbar_init(smem_u32(&ctl.scan_empty[i]), kProducerWarps);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(smem_u32(&ctl.sready[i]), 1);
        }
        mbar_init(smem_u32(&ctl.pfull), 1);
        mbar_init(smem_u32(&ctl.pempty), kDrainWarps);
        mbar_init(smem_u32(&ctl.xfull), 1);
        mbar_init(smem_u32(&ctl.xempty), kDrainWarps);
        mbar_init(smem_u32(&ctl.strip_free), 1);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        fence_mbar_init();
    }
    __syncthreads();
    fence_before();
    __syncthreads();
    fence_after();

    if (warp < kDrainWarps) {
        // ---- drain warps: running sums, outputs ----------------------------------------------
        const int quarter = warp & 3;
        const int slice = warp >> 2;
        const int r = kB - 1 - (quarter * 32 + lane);
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(slice * kCols);
        float acc[kCols];
#pragma unroll
        for (int i = 0; i < kCols; ++i) {
            acc[i] = 0.0f;
        }
        auto drain = [&](uint32_t col) {
            fence_after();
#pragma unroll
            for (int c16 = 0; c16 < kCols / 16; ++c16) {
                uint32_t t[16];
                tmem_ld16(lane_addr + col + static_cast<uint32_t>(c16 * 16), t);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    acc[c16 * 16 + i] += __uint_as_float(t[i]);
                }
            }
            fence_before();
            __syncwarp();
        };
        bool ok = true;
        int g = 0;   // H groups drained so far
        for (int k = 0; k < my_items && ok && !*abort; ++k) {
            // Item k's description (published with its scale before its first stage, so
            // before any of its MMAs: no wait in practice). Read from shared memory rather
            // than looked up in the capture table, which kept too many registers live.
            if (!mbar_wait_bounded(smem_u32(&ctl.sready[k & 3]), (k >> 2) & 1, fault,
                                   kFaultScale, abort)) {
                break;
            }
            const int per_tile = *reinterpret_cast<volatile int*>(&ctl.item_groups[k & 3]);
            for (int gi = 0; gi < per_tile; ++gi, ++g) {
                if (!mbar_wait_bounded(smem_u32(&ctl.pfull), g & 1, fault, kFaultAccumFull,
                                       abort)) {
                    ok = false;
                    break;
                }
                drain(0);
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.pempty));
                }
            }
            if (!ok ||
                !mbar_wait_bounded(smem_u32(&ctl.xfull), k & 1, fault, kFaultAccumFull, abort)) {
                break;
            }
            drain(kXCol);
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.xempty));
            }
            // Slot k % 4 is rewritten only for item k + 4, which needs this drain finished.
            const int shift = -*reinterpret_cast<volatile int*>(&ctl.shift[k & 3]);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            float2* const y = *reinterpret_cast<float2* volatile*>(&ctl.item_y[k & 3]);
            const long long n_out = *reinterpret_cast<volatile long long*>(&ctl.item_n[k & 3]);
            const long long jb0 = *reinterpret_cast<volatile long long*>(&ctl.item_block0[k & 3]) +
                                  slice * (kCols / 2);
#pragma unroll
            for (int b = 0; b < kCols / 2; ++b) {
                const long long o = (jb0 + b) * kB + r;
                if (o < n_out) {
                    y[o] = make_float2(acc[2 * b] * fa * fb, acc[2 * b + 1] * fa * fb);
                }
                acc[2 * b] = 0.0f;
                acc[2 * b + 1] = 0.0f;
            }
        }
    } else if (warp < kFirstProducerWarp + kProducerWarps) {
        // ---- producers: tap strips, scales, operand stages, copies ---------------------------
        const int pw = warp - kFirstProducerWarp;
        const int ptid = static_cast<int>(threadIdx.x) - kFirstProducerWarp * 32;
        int ex_even = 0;            // sample scale exponents of even and odd items
        int ex_odd = 0;
        int eh = 0;                 // tap scale exponent of capture eh_cap
        int eh_cap = -1;
        int switches = 0;           // tap strips rebuilt after the first (strip_free phases)
        int tmax_uses = 0;
        uint32_t next_max = 0;
        CapCursor cp;               // capture of the K-step being converted
        cursor_load(p, cap_first, cp);
        CapCursor cs = cp;          // capture of the scan slice being read (one item ahead)
        // Copies, issued by producer thread 0: raw K-step copies kRaw ahead, scan slices
        // sbufs - 2 ahead, each capture's fields in the thread's own cursors.
        CapCursor cr = cp;          // capture of the next raw copy
        CapCursor cq = cp;          // capture of the next scan slice (one item ahead)
        // The last capture whose tensor maps this thread has fenced (its captures are met in
        // increasing order from cap_first).
        int fenced = cap_first - 1;
        auto acquire_maps = [&](int cursor) {
            if (p.maps_global) {
                for (; fenced < cursor; ++fenced) {
                    tmap_acquire(p.xmap + fenced + 1);
                    tmap_acquire(p.smap + fenced + 1);
                }
            }
        };
        // Raw copy of K-step u into raw slot `slot`: item u / 8, floats 32 (u % 8) .. of its
        // window (rows from block tile * kNB - C).
        auto issue_raw = [&](int u, int slot) {
            const int k = u / kStagesPerTile;
            cursor_seek(p, first_item + k, cr);
            acquire_maps(cr.idx);
            const uint32_t bar = smem_u32(&ctl.raw_full[slot]);
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(kNB + cr.C) * 128u);
            tma_load_2d(sbase + lay.raw0 + static_cast<uint32_t>(slot) * lay.raw, p.xmap + cr.idx,
                        32 * (u % kStagesPerTile), (first_item + k - cr.item0) * kNB - cr.C, bar);
        };
        // Scan slice q: item q / 8 + 1's window rows (q % 8) srows .. + srows.
        auto issue_scan = [&](int q) {
            const int kn = q / kStagesPerTile + 1;
            cursor_seek(p, first_item + kn, cq);
            acquire_maps(cq.idx);
            const int srows = (kNB + cq.C + kStagesPerTile - 1) / kStagesPerTile;
            const uint32_t bar = smem_u32(&ctl.scan_full[q % sbufs]);
            mbar_arrive_expect_tx(bar, static_cast<uint32_t>(srows) * 1024u);
            tma_load_2d(sbase + lay.scan0 + static_cast<uint32_t>(q % sbufs) * lay.scan,
                        p.smap + cq.idx, 0,
                        (first_item + kn - cq.item0) * kNB - cq.C + (q % kStagesPerTile) * srows,
                        bar);
        };

        // Max of |samples| of capture c in [s, s + 2) clipped to hi_s.
        auto load_pair = [&](const BatchCap& c, long long s, long long hi_s) -> uint32_t {
            if (s + 1 < hi_s) {
                return absmax4(__ldg(reinterpret_cast<const float4*>(c.x + s)));
            }
            if (s < hi_s) {
                const float2 w2 = __ldg(c.x + s);
                return max(absbits(w2.x), absbits(w2.y));
            }
            return 0u;
        };
        // Max over the producers of a per-thread value (all producers call it together).
        auto producers_max = [&](uint32_t m, uint32_t (&slots)[2][kProducerWarps], int use) {
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            if (lane == 0) {
                slots[use & 1][pw] = m;
            }
            asm volatile("bar.sync 1, %0;" ::"n"(kProducers) : "memory");
            uint32_t t = 0;
#pragma unroll
            for (int w = 0; w < kProducerWarps; ++w) {
                t = max(t, slots[use & 1][w]);
            }
            return t;
        };
        // Tap scale exponent of capture ci (once per capture, when its first tile's scale is
        // published).
        auto tap_exponent = [&](int ci) {
            const BatchCap& c = p.cap[ci];
            uint32_t m = 0;
            for (int i = ptid; i < c.num_taps; i += kProducers) {
                m = max(m, absbits(__ldg(c.taps + i)));
            }
            eh = scale_exponent(producers_max(m, ctl.tmaxw, tmax_uses++));
            eh_cap = ci;
        };
        // Item k's sample scale from its window maximum m, and its output shift ex + eh.
        auto reduce_scale = [&](int k, uint32_t m, int ci) {
            const uint32_t tmax = producers_max(m, ctl.pmax, k);
            if (ci != eh_cap) {
                tap_exponent(ci);
            }
            const int ex = min(scale_exponent(tmax), 127);
            if (k & 1) {
                ex_odd = ex;
            } else {
                ex_even = ex;
            }
            if (ptid == 0) {
                const BatchCap& c = p.cap[ci];
                ctl.shift[k & 3] = ex + eh;
                ctl.item_y[k & 3] = c.y;
                ctl.item_n[k & 3] = c.n;
                ctl.item_block0[k & 3] = static_cast<long long>(first_item + k - c.item0) * kNB;
                ctl.item_groups[k & 3] = h_groups(c.C + 1, S).per_tile;
                mbar_arrive(smem_u32(&ctl.sready[k & 3]));
            }
        };
        // The tap strip of capture ci, scaled by 2^eh (eh of ci).
        auto build_strip = [&](int ci) {
            const BatchCap& c = p.cap[ci];
            const float fa = exp2i(eh / 2);
            const float fb = exp2i(eh - eh / 2);
            const int dmax = (c.C + 1) * kB - 1;
            const int pairs = (16 * c.C + 31) * 32;
            for (int i = ptid; i < pairs; i += kProducers) {
                const int t = i >> 5;
                const int q = (i >> 2) & 7;
                const int e = (i & 3) * 2;
                const int i0 = dmax - 8 * t - q - e;
                const int i1 = i0 - 1;
                const float v0 = (i0 >= 0 && i0 < c.num_taps) ? __ldg(c.taps + i0) * fa * fb : 0.0f;
                const float v1 = (i1 >= 0 && i1 < c.num_taps) ? __ldg(c.taps + i1) * fa * fb : 0.0f;
                uint32_t hi, lo;
                split2(v0, v1, hi, lo);
                const uint32_t off = static_cast<uint32_t>(t) * 128u + q * 16u + e * 2u;
                sts32(sbase + lay.taps_hi + off, hi);
                sts32(sbase + lay.taps_lo + off, lo);
            }
            // Made visible to the MMAs by the fence before this K-step's full arrival.
        };
        // The geometry of the item whose window the scan slices cover, computed at its first
        // slice.
        int sc_item = -1;
        int sc_rows = 0;          // window rows
        int sc_srows = 0;         // rows per slice
        long long sc_full = 0;    // full blocks of the capture
        long long sc_tail = 0;    // window row of the capture's partial block
        // Scan slice q (item q / 8 + 1), copied by TMA sbufs - 1 K-steps earlier.
        auto consume_slice = [&](int q) -> bool {
            const int qb = q % sbufs;
            if (!mbar_wait_bounded(smem_u32(&ctl.scan_full[qb]), (q / sbufs) & 1, fault,
                                   kFaultTileLoad, abort)) {
                return false;
            }
            const int k = q / kStagesPerTile + 1;
            if (k != sc_item) {
                sc_item = k;
                cursor_seek(p, first_item + k, cs);
                sc_rows = kNB + cs.C;
                sc_srows = (sc_rows + kStagesPerTile - 1) / kStagesPerTile;
                sc_full = cs.n / kB;
                sc_tail = sc_full - (static_cast<long long>(first_item + k - cs.item0) * kNB - cs.C);
            }
            const int r0 = (q % kStagesPerTile) * sc_srows;
            const uint32_t buf = sbase + lay.scan0 + static_cast<uint32_t>(qb) * lay.scan;
            const int quads = min(sc_srows, sc_rows - r0) * 64;   // sample pairs in the window
            uint32_t m = next_max;
#pragma unroll 4
            for (int f = ptid; f < quads; f += kProducers) {
                m = max(m, absmax4(lds128(buf + static_cast<uint32_t>(f) * 16u)));
            }
            // The capture's partial last block lies outside its tensor map.
            const long long tail_row = sc_tail - r0;
            if (tail_row >= 0 && tail_row * 64 < quads && ptid < 64) {
                m = max(m, load_pair(p.cap[cs.idx], sc_full * kB + 2 * ptid, cs.n));
            }
            next_max = m;
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.scan_empty[qb]));
            }
            if (q % kStagesPerTile == kStagesPerTile - 1) {
                reduce_scale(k, next_max, cs.idx);
                next_max = 0;
            }
            return true;
        };
        // The capture of the K-steps being converted, as loop invariants of a segment (the
        // block's K-steps of one capture).
        int seg_C = 0;
        int seg_rows = 0;
        long long seg_full = 0;    // full blocks of the capture (rows its tensor maps cover)
        long long seg_tile0 = 0;   // tile, within the capture, of the block's item 0
        long long seg_n = 0;
        const float2* seg_x = nullptr;
        // Producing K-step v: finish scan slice v - 1, convert the raw samples, queue step
        // v + kRaw's raw copy and scan slice v + sbufs - 2.
        auto produce = [&](int v) -> bool {
            if (v >= 1 && v - 1 < scan_slices && !consume_slice(v - 1)) {
                return false;
            }
            const int k = v / kStagesPerTile;
            const int st = v % kStagesPerTile;
            const long long j0 = (seg_tile0 + k) * kNB;
            const int ex = (k & 1) ? ex_odd : ex_even;
            const float fs = exp2_exact(ex);   // ex in [-113, 127]: exact scaling
            const f32x2 fs2 = pack2(fs, fs);
            const int slot = v % S;
            const int rslot = v % kRaw;
            if (!mbar_wait_bounded(smem_u32(&ctl.empty[slot]), ((v / S) & 1) ^ 1, fault,
                                   kFaultStageEmpty, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.raw_full[rslot]), (v / kRaw) & 1, fault,
                                   kFaultTileLoad, abort)) {
                return false;
            }
            const uint32_t stage = sbase + lay.stages0 + static_cast<uint32_t>(slot) * lay.stage;
            const uint32_t raw = sbase + lay.raw0 + static_cast<uint32_t>(rslot) * lay.raw;
            const long long tail_rel = seg_full - (j0 - seg_C);
            const int b_tail = tail_rel >= 0 && tail_rel < seg_rows ? static_cast<int>(tail_rel) : -1;
            static_assert(kProducers % 8 == 0, "producer stride");
            const int q = ptid & 7;
            const uint32_t elem_off = static_cast<uint32_t>(q >> 2) * lay.pitch +
                                      static_cast<uint32_t>(q & 3) * 4u;
#pragma unroll 2
            for (int b = ptid >> 3; b < seg_rows; b += kProducers / 8) {
                const int f = 8 * b + q;
                float4 v4;
                if (b != b_tail) {
                    v4 = lds128(raw + static_cast<uint32_t>(f) * 16u);  // zero outside [0, n)
                } else {
                    const long long sidx = seg_full * kB + 16 * st + 2 * q;
                    v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (sidx + 1 < seg_n) {
                        v4 = __ldg(reinterpret_cast<const float4*>(seg_x + sidx));
                    } else if (sidx < seg_n) {
                        const float2 w2 = __ldg(seg_x + sidx);
                        v4.x = w2.x;
                        v4.y = w2.y;
                    }
                }
                const float2 s0 = unpack2(mul2(pack2(v4.x, v4.y), fs2));
                const float2 s1 = unpack2(mul2(pack2(v4.z, v4.w), fs2));
                uint32_t re_hi, re_lo, im_hi, im_lo;
                split2(s0.x, s1.x, re_hi, re_lo);
                split2(s0.y, s1.y, im_hi, im_lo);
                const uint32_t row_re = elem_off + static_cast<uint32_t>(2 * b) * 16u;
                sts32(stage + row_re, re_hi);
                sts32(stage + row_re + 16u, im_hi);
                sts32(stage + lay.split + row_re, re_lo);
                sts32(stage + lay.split + row_re + 16u, im_lo);
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.full[slot]));
                mbar_arrive(smem_u32(&ctl.raw_empty[rslot]));
            }
            if (ptid == 0) {
                if (v + kRaw < my_steps) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.raw_empty[rslot]), (v / kRaw) & 1,
                                           fault, kFaultStageEmpty, abort)) {
                        return false;
                    }
                    issue_raw(v + kRaw, rslot);
                }
                const int qn = v + sbufs - 2;
                if (qn < scan_slices) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.scan_empty[qn % sbufs]),
                                           ((qn / sbufs) & 1) ^ 1, fault, kFaultStageEmpty,
                                           abort)) {
                        return false;
                    }
                    issue_scan(qn);
                }
            }
            return true;
        };

        if (ptid == 0) {
            for (int u = 0; u < kRaw && u < my_steps; ++u) {
                issue_raw(u, u);
            }
            for (int q = 0; q < sbufs - 2 && q < scan_slices; ++q) {
                issue_scan(q);
            }
        }
        // Item 0: its capture's tap scale and strip, its scale from its whole window.
        {
            const BatchCap& c = p.cap[cp.idx];
            const long long j0 = static_cast<long long>(first_item - c.item0) * kNB;
            const long long win0 = (j0 - c.C) * kB;
            const long long lo0 = win0 > 0 ? win0 : 0;
            const long long hi0 = (j0 + kNB) * kB < c.n ? (j0 + kNB) * kB : c.n;
            const long long pairs = (hi0 - lo0 + 1) / 2;
            uint32_t m = 0;
            for (long long base = 0; base < pairs; base += 8 * kProducers) {
                uint32_t part[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const long long idx = base + ptid + i * kProducers;
                    part[i] = idx < pairs ? load_pair(c, lo0 + 2 * idx, hi0) : 0u;
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    m = max(m, part[i]);
                }
            }
            reduce_scale(0, m, cp.idx);
            build_strip(cp.idx);
        }
        bool ok = true;
        int v = 0;
        while (v < my_steps && ok && !*abort) {
            if (cursor_seek(p, first_item + v / kStagesPerTile, cp)) {
                // A new capture: every MMA that reads the old strip has completed before it is
                // overwritten.
                if (!mbar_wait_bounded(smem_u32(&ctl.strip_free), switches & 1, fault,
                                       kFaultStageEmpty, abort)) {
                    break;
                }
                ++switches;
                // The strip is scaled by the new capture's tap exponent (all producers together;
                // the scale of the capture's first item, published later, uses the same).
                if (eh_cap != cp.idx) {
                    tap_exponent(cp.idx);
                }
                build_strip(cp.idx);
            }
            seg_C = cp.C;
            seg_rows = kNB + cp.C;
            seg_full = cp.n / kB;
            seg_tile0 = first_item - cp.item0;
            seg_n = cp.n;
            seg_x = p.cap[cp.idx].x;
            const int end_item = min(my_items, cp.end - first_item);
            for (; v < end_item * kStagesPerTile && ok && !*abort; ++v) {
                ok = produce(v);
            }
        }
    } else if (warp == kMmaWarp && lane == 0) {
        // ---- MMA issuer (one thread), as in fir_tc.cu, per item's capture -------------------
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        const uint32_t h_acc = tmem;
        const uint32_t x_acc = tmem + kXCol;
        CapCursor cm;
        cursor_load(p, cap_first, cm);
        int ready = 0;
        int g = 0;
        bool stop = false;
        // The capture's chunk count, H groups and descriptor bases, recomputed at a switch.
        int grp_cap = -1;
        int P = 0;
        HGroups grp{};
        uint32_t a_hi0 = 0;
        uint32_t a_lo0 = 0;
        uint32_t b_base = 0;
        for (int k = 0; k < my_items && !stop && !*abort; ++k) {
            cursor_seek(p, first_item + k, cm);
            if (cm.idx != grp_cap) {
                grp_cap = cm.idx;
                const int C = cm.C;
                P = C + 1;
                grp = h_groups(P, S);
                a_hi0 = ((sbase + lay.taps_hi) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
                a_lo0 = ((sbase + lay.taps_lo) >> 4) + static_cast<uint32_t>(16 * C) * 8u;
                b_base = ((sbase + lay.stages0) >> 4) + static_cast<uint32_t>(2 * C);
            }
            for (int gi = 0; gi < grp.per_tile && !stop; ++gi, ++g) {
                int st0, st1, c0, c1;
                h_group_range(grp, P, gi, st0, st1, c0, c1);
                if (!mbar_wait_bounded(smem_u32(&ctl.pempty), (g & 1) ^ 1, fault,
                                       kFaultAccumEmpty, abort)) {
                    stop = true;
                    break;
                }
                fence_after();
                uint32_t acc = 0;
                for (int st = st0; st < st1; ++st) {
                    const int u = k * kStagesPerTile + st;
                    const int slot = u % S;
                    if (u >= ready) {
                        if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (u / S) & 1, fault,
                                               kFaultStageFull, abort)) {
                            stop = true;
                            break;
                        }
                        fence_after();
                        ready = u + 1;
                    }
                    unsigned long long da =
                        a_desc | (a_hi0 + static_cast<uint32_t>(2 * st - 16 * c0) * 8u);
                    unsigned long long db =
                        b_desc | (b_base + static_cast<uint32_t>(slot) * stage_units -
                                  static_cast<uint32_t>(2 * c0));
                    int c = c0;
                    if (acc == 0) {
                        mma_f16<kIdesc>(h_acc, da, db, 0u);
                        acc = 1;
                        da -= 128;
                        db -= 2;
                        ++c;
                    }
                    for (; c < c1; ++c) {
                        mma_f16_acc<kIdesc>(h_acc, da, db);
                        da -= 128;
                        db -= 2;
                    }
                }
                if (stop) {
                    break;
                }
                mma_commit(smem_u32(&ctl.pfull));
                if (gi == 0) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.xempty), (k & 1) ^ 1, fault,
                                           kFaultAccumEmpty, abort)) {
                        stop = true;
                        break;
                    }
                    fence_after();
                }
                acc = gi == 0 ? 0u : 1u;
                for (int st = st0; st < st1; ++st) {
                    const int slot = (k * kStagesPerTile + st) % S;
                    const uint32_t off = static_cast<uint32_t>(2 * st - 16 * c0) * 8u;
                    unsigned long long dah = a_desc | (a_hi0 + off);
                    unsigned long long dal = a_desc | (a_lo0 + off);
                    unsigned long long dbh =
                        b_desc | (b_base + static_cast<uint32_t>(slot) * stage_units -
                                  static_cast<uint32_t>(2 * c0));
                    unsigned long long dbl = dbh + split_units;
                    int c = c0;
                    if (acc == 0) {
                        mma_f16<kIdesc>(x_acc, dah, dbl, 0u);
                        mma_f16_acc<kIdesc>(x_acc, dal, dbh);
                        acc = 1;
                        dah -= 128;
                        dal -= 128;
                        dbh -= 2;
                        dbl -= 2;
                        ++c;
                    }
                    for (; c < c1; ++c) {
                        mma_f16_acc<kIdesc>(x_acc, dah, dbl);
                        mma_f16_acc<kIdesc>(x_acc, dal, dbh);
                        dah -= 128;
                        dal -= 128;
                        dbh -= 2;
                        dbl -= 2;
                    }
                    if (c1 == P) {
                        mma_commit(smem_u32(&ctl.empty[slot]));
                    }
                }
            }
            if (stop) {
                break;
            }
            mma_commit(smem_u32(&ctl.xfull));
            // The strip of this capture is free once these MMAs complete.
            if (k + 1 < my_items && first_item + k + 1 >= cm.end) {
                mma_commit(smem_u32(&ctl.strip_free));
            }
        }
        mma_commit(smem_u32(&ctl.teardown));
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
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

// True on every thread of plain group `id` if `v` is true on all of them (one barrier).
__device__ __forceinline__ bool group_all(bool v, uint32_t id)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(v)), "r"(id), "n"(kPlainThreads)
        : "memory");
    return r != 0;
}

// Plain tiles t0 .. t1 - 1 of the work list, by plain_groups groups of 256 threads (group g
// takes tiles t0 + g, t0 + g + groups, ...), each with its own shared-memory region and named
// barrier: the plain kernel's tile function, so the same bits as fir_plain_kernel.
__device__ __forceinline__ void batch_plain_tiles(const BatchView& p, int t0, int t1,
                                                  unsigned char* smem)
{
    const int group = static_cast<int>(threadIdx.x) / kPlainThreads;
    if (group >= p.plain_groups) {
        return;
    }
    const int gtid = static_cast<int>(threadIdx.x) % kPlainThreads;
    unsigned char* region = smem + 1024 + static_cast<uint32_t>(group) * p.plain_region;
    const PlainGroupSync sync{static_cast<uint32_t>(2 + group)};
    if (p.plain_region >= 2 * p.plain_slot) {
        // Two slots: each tile's copy overlaps the previous tile's computation.
        int c = 0;
        auto source = [&](int i) {
            const int t = t0 + group + i * p.plain_groups;
            while (c + 1 < p.pcount && p.pcap[c + 1].tile0 <= t) {
                ++c;
            }
            const PlainCapDev& pc = p.pcap[c];
            return PlainTileRef{pc.x, pc.taps, pc.y, pc.n, pc.num_taps,
                                static_cast<long long>(t - pc.tile0)};
        };
        const int count = t1 - t0 > group ? (t1 - t0 - group + p.plain_groups - 1) / p.plain_groups
                                          : 0;
        fir_plain_group_tiles(source, count, region, p.plain_slot, &g_fault_fir_batch, gtid, sync,
                              [&](bool v) { return group_all(v, sync.id); });
        return;
    }
    uint32_t phase = 0;
    bool init = true;
    int c = 0;
    for (int t = t0 + group; t < t1; t += p.plain_groups) {
        while (c + 1 < p.pcount && p.pcap[c + 1].tile0 <= t) {
            ++c;
        }
        const PlainCapDev& pc = p.pcap[c];
        const bool ok = fir_plain_tile<0>(pc.x, pc.taps, pc.y, pc.n, pc.num_taps, t - pc.tile0,
                                          region, &g_fault_fir_batch, gtid, sync, phase, init);
        init = false;
        if (!group_all(ok, sync.id)) {
            break;   // a copy gave up (fault recorded): the whole group stops together
        }
    }
}

// The window phase that reaches back C blocks runs with eight operand stages (converted four
// K-steps at a time, as the single-capture kernel: four stages convert two at a time, measured
// 3.2 - 3.8 SM-us per tile at C = 1 against 3.0), beside three windows and, where they fit, two
// tap-strip slots (the next capture's strip built while the last one's MMAs run); at C = 2, 3
// one slot, rebuilt once the capture's MMAs are done.
__host__ __device__ constexpr int win_stages(int) { return 8; }
__host__ __device__ constexpr int win_strips(int C) { return C == 1 ? 2 : 1; }

// One window phase: the block's items of the captures that reach back C blocks.
template <int C>
__device__ __forceinline__ void batch_window_items(const BatchView& v, unsigned char* smem,
                                                   uint32_t tmem)
{
    if (v.wcount[C - 1] == 0) {
        return;
    }
    const int w0 = v.cta_win[C - 1][blockIdx.x];
    const int w1 = v.cta_win[C - 1][blockIdx.x + 1];
    if (w1 <= w0) {
        return;   // uniform across the block
    }
    const tcw::TcwListSrc src{v.wcap[C - 1], v.wmap[C - 1], v.wcount[C - 1], w0, w1 - w0};
    tcw::Ctrl& wctl = *reinterpret_cast<tcw::Ctrl*>(smem + v.win_ctl);
    tcw::tcw_pipeline<C, 0, win_stages(C), tcw::TcwListSrc, win_strips(C)>(src, smem, wctl, tmem,
                                                                        &g_fault_fir_batch);
    if (threadIdx.x == 0) {
        tcw::tcw_release<win_stages(C)>(wctl);
    }
    __syncthreads();
}

template <int S>
__device__ __forceinline__ void batch_body(const BatchView& v, unsigned char* smem)
{
    static_assert(kThreads >= tcw::kThreads, "the window pipeline's roles fit the block");
    // Tensor memory for every phase, taken once (a block relinquishes the right to allocate
    // with its first allocation); the base travels through the control block's last word.
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 1020);
    const int warp = threadIdx.x >> 5;
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(tmem_slot), kTmemCols);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    __syncthreads();   // read before any phase writes shared memory
    const int first_item = v.cta_item[blockIdx.x];
    const int my_items = v.cta_item[blockIdx.x + 1] - first_item;
    if (my_items > 0) {
        batch_tc_items<S>(v, first_item, my_items, smem, tmem);
    }
    batch_window_items<1>(v, smem, tmem);
    batch_window_items<2>(v, smem, tmem);
    batch_window_items<3>(v, smem, tmem);
    if (v.plain_groups > 0) {
        const int t0 = v.cta_plain[blockIdx.x];
        const int t1 = v.cta_plain[blockIdx.x + 1];
        if (t1 > t0) {
            batch_plain_tiles(v, t0, t1, smem);
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == kMmaWarp) {
        tmem_dealloc(tmem, kTmemCols);
    }
}

// rfx_fir_batch_launch: the work list in the kernel parameters (tensor-core captures only).
template <int S>
__global__ void __launch_bounds__(kThreads, 1)
fir_batch_kernel(const __grid_constant__ BatchParams p)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const BatchView v{p.cap,   p.xmap,  p.smap, p.cta_item, nullptr, nullptr, p.count,
                      0,       p.cmax,  p.sbufs, 0,         0u,      0u,      0,
                      {},      {},      {},      {},        0u};
    batch_body<S>(v, smem);
}

// A batch plan: the work list in device memory, tensor-core and plain captures in one launch.
template <int S>
__global__ void __launch_bounds__(kThreads, 1)
fir_batch_list_kernel(const __grid_constant__ BatchView v)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    batch_body<S>(v, smem);
}

namespace {

// Splits the items of `caps` into `parts` contiguous ranges of about equal cost (every range
// non-empty; parts <= total_items).
void partition(const std::vector<BatchCap>& caps, int total_items, int parts, int* cta_item)
{
    std::vector<double> prefix(total_items + 1, 0.0);
    for (const BatchCap& c : caps) {
        // Measured on GB300 (the single-capture kernel, same pipeline): a tile costs about the
        // same whatever its filter from 63 to 1025 taps (15.2 and 15.7 us per tile and SM).
        const double per_tile = 1.0 + 0.007 * static_cast<double>(c.C + 1);
        for (int t = 0; t < c.tiles; ++t) {
            prefix[c.item0 + t + 1] = per_tile;
        }
    }
    for (int i = 0; i < total_items; ++i) {
        prefix[i + 1] += prefix[i];
    }
    cta_item[0] = 0;
    for (int b = 1; b < parts; ++b) {
        const double target = prefix[total_items] * b / parts;
        int item = static_cast<int>(std::lower_bound(prefix.begin(), prefix.end(), target) -
                                    prefix.begin());
        item = std::max(item, cta_item[b - 1] + 1);
        item = std::min(item, total_items - (parts - b));
        cta_item[b] = item;
    }
    cta_item[parts] = total_items;
}

template <int S>
cudaError_t launch_batch(const BatchParams& params, int grid, const Layout& lay,
                         cudaStream_t stream)
{
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    cudaError_t err = cudaFuncSetAttribute(fir_batch_kernel<S>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    fir_batch_kernel<S><<<grid, kThreads, bytes, stream>>>(params);
    return cudaGetLastError();
}

}  // namespace

bool fir_batch_supported(int num_taps)
{
    return fir_tc_supported(num_taps) &&
           batch_layout((num_taps + kB - 2) / kB, 2, 2).bytes <= 227u * 1024u;
}

cudaError_t fir_batch_tc_launch(const rfx_fir_capture* captures, int count, cudaStream_t stream)
{
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    sms = std::min(sms, kBatchCtas);
    // Captures the tensor-core kernel takes go into the work list; the rest (one tap, shorter
    // than a block, or taps beyond the shared-memory budget) run the plain kernel, in order.
    std::vector<BatchCap> caps;
    std::vector<CUtensorMap> xmaps;
    std::vector<CUtensorMap> smaps;
    for (int i = 0; i < count; ++i) {
        const rfx_fir_capture& c = captures[i];
        if (c.num_samples == 0) {
            continue;
        }
        if (c.num_samples < kB || !fir_batch_supported(c.num_taps)) {
            err = fir_plain_launch(c.x, c.taps, c.y, c.num_samples, c.num_taps, stream);
            if (err != cudaSuccess) {
                return err;
            }
            continue;
        }
        BatchCap b{};
        b.x = static_cast<const float2*>(c.x);
        b.y = static_cast<float2*>(c.y);
        b.taps = c.taps;
        b.n = c.num_samples;
        b.num_taps = c.num_taps;
        b.C = (c.num_taps + kB - 2) / kB;
        const long long blocks = (c.num_samples + kB - 1) / kB;
        b.tiles = static_cast<int>((blocks + kNB - 1) / kNB);
        // x as rows of 256 floats (full 128-sample blocks only); boxes of one K-step's 32
        // floats by the window's rows, and of whole rows by a scan slice's rows.
        const Geo g = geo_of(b.C, b.n);
        CUtensorMap xm;
        CUtensorMap sm;
        err = encode_rows(&xm, c.x, 4, b.n / kB, 2 * kB, 32, static_cast<uint32_t>(g.rows));
        if (err == cudaSuccess) {
            err = encode_rows(&sm, c.x, 4, b.n / kB, 2 * kB, 2 * kB,
                              static_cast<uint32_t>(g.srows));
        }
        if (err != cudaSuccess) {
            return err;
        }
        caps.push_back(b);
        xmaps.push_back(xm);
        smaps.push_back(sm);
    }
    for (std::size_t first = 0; first < caps.size(); first += kBatchCaps) {
        const std::size_t chunk = std::min<std::size_t>(kBatchCaps, caps.size() - first);
        std::vector<BatchCap> part(caps.begin() + first, caps.begin() + first + chunk);
        int items = 0;
        int cmax = 0;
        for (BatchCap& b : part) {
            b.item0 = items;
            items += b.tiles;
            cmax = std::max(cmax, b.C);
        }
        const int grid = std::min(items, sms);
        BatchParams* params = new BatchParams{};
        for (std::size_t i = 0; i < chunk; ++i) {
            params->cap[i] = part[i];
            params->xmap[i] = xmaps[first + i];
            params->smap[i] = smaps[first + i];
        }
        params->count = static_cast<int>(chunk);
        params->cmax = cmax;
        partition(part, items, grid, params->cta_item);
        // The deep scan ring first, then the most operand stages that fit.
        err = cudaErrorInvalidValue;
        bool launched = false;
        for (int sbufs = kScanBufsMax; sbufs >= 2 && !launched; sbufs -= 2) {
            params->sbufs = sbufs;
            for (int stages : {6, 4, 2}) {
                const Layout lay = batch_layout(cmax, stages, sbufs);
                if (lay.bytes > 227u * 1024u) {
                    continue;
                }
                err = stages == 6   ? launch_batch<6>(*params, grid, lay, stream)
                      : stages == 4 ? launch_batch<4>(*params, grid, lay, stream)
                                    : launch_batch<2>(*params, grid, lay, stream);
                launched = true;
                break;
            }
        }
        delete params;
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
}

// ---- batch plans: the work list in device memory, one launch ---------------------------------

namespace {

// Cost of a work unit in microseconds of one SM, for the partition. Measured on GB300 with this
// kernel (batch plans of each tap count of the 256-capture workload alone, CUDA-graph replay):
// a long-filter tile of 96 blocks takes 16.4 SM-us at 511 taps (C = 4) and 18.7 at 1025
// (C = 8); a plain tile of 2304 outputs 1.66, 2.27, 3.90, 6.54, 12.6 and 24.7 SM-us at 31, 63,
// 127, 255, 511 and 1025 taps.
double tc_tile_us(int C) { return 13.5 + 0.58 * static_cast<double>(C + 1); }
double plain_tile_us(int num_taps) { return 1.0 + 0.0233 * static_cast<double>(num_taps); }
// A resident-window tile of 48 blocks (batch plans as above: 3.0, 2.9 and 3.6 SM-us at 31, 63
// and 127 taps, 4.2 at 255; C = 3 scaled from single captures of 2^24 samples, 2.98, 3.82 and
// 4.69 SM-us for C = 1, 2, 3), and the tap strip built per capture.
double win_tile_us(int C) { return C == 1 ? 3.1 : C == 2 ? 4.2 : 5.2; }
constexpr double kWinStripUs = 1.0;

constexpr int kPlainGroupsMax = kThreads / kPlainThreads;   // 3
constexpr uint32_t kSmemMax = 227u * 1024u;

uint32_t align_up(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct BatchPlan {
    void* dev = nullptr;
    BatchView view{};
    int grid = 0;
    int stages = 0;
    uint32_t smem = 0;
    int tc_caps = 0;
    int plain_caps = 0;
};

void fir_batch_plan_free(BatchPlan* plan)
{
    if (plan != nullptr) {
        cudaFree(plan->dev);
        delete plan;
    }
}

void fir_batch_plan_counts(const BatchPlan* plan, int* tc_captures, int* plain_captures,
                           int* launches)
{
    *tc_captures = plan->tc_caps;
    *plain_captures = plan->plain_caps;
    *launches = plan->grid > 0 ? 1 : 0;
}

cudaError_t fir_batch_plan_make(int impl, const rfx_fir_capture* captures, int count,
                                BatchPlan** out)
{
    *out = nullptr;
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    // Which kernel takes each capture: the tensor-core pipeline where the call's implementation
    // (auto: the tuned table) puts it and the batch kernel can take it, the plain tile otherwise.
    std::vector<BatchCap> tc;
    std::vector<CUtensorMap> xmaps, smaps;
    std::vector<PlainCapDev> pl;
    // Resident-window captures by blocks reached back (C = 1, 2, 3), their maps and costs.
    std::vector<tcw::WinCapture> wc[tcw::kCMax];
    std::vector<CUtensorMap> wm[tcw::kCMax];
    std::vector<double> wcost[tcw::kCMax];
    std::vector<double> cost;       // per work unit: tensor-core items, then plain tiles
    int kmax_plain = 0;
    int cmax = 0;
    int items = 0;
    int ptiles = 0;
    std::vector<double> plain_cost;
    for (int i = 0; i < count; ++i) {
        const rfx_fir_capture& c = captures[i];
        if (c.num_samples == 0) {
            continue;
        }
        const int want =
            impl == RFX_FIR_AUTO ? tuned_fir_batch_impl(c.num_taps, c.num_samples) : impl;
        const bool use_win = want == RFX_FIR_TC && c.num_samples >= kB &&
                             fir_tcw_supported(c.num_taps);
        const bool use_tc = !use_win && want == RFX_FIR_TC && c.num_samples >= kB &&
                            fir_batch_supported(c.num_taps);
        if (use_win) {
            const int C = (c.num_taps + kB - 2) / kB;
            std::vector<tcw::WinCapture>& list = wc[C - 1];
            const int item0 = list.empty() ? 0 : list.back().item0 +
                                                     static_cast<int>(((list.back().n + kB - 1) / kB +
                                                                       tcw::kNB - 1) / tcw::kNB);
            list.push_back(tcw::WinCapture{c.x, static_cast<float2*>(c.y), c.taps, c.num_samples,
                                           c.num_taps, item0});
            CUtensorMap m;
            err = encode_rows(&m, c.x, 4, c.num_samples / kB, 2 * kB, 2 * kB,
                              static_cast<uint32_t>(tcw::kNB + C));
            if (err != cudaSuccess) {
                return err;
            }
            wm[C - 1].push_back(m);
            const int tiles = static_cast<int>(((c.num_samples + kB - 1) / kB + tcw::kNB - 1) /
                                               tcw::kNB);
            for (int t = 0; t < tiles; ++t) {
                wcost[C - 1].push_back(win_tile_us(C) + (t == 0 ? kWinStripUs : 0.0));
            }
        } else if (use_tc) {
            BatchCap b{};
            b.x = static_cast<const float2*>(c.x);
            b.y = static_cast<float2*>(c.y);
            b.taps = c.taps;
            b.n = c.num_samples;
            b.num_taps = c.num_taps;
            b.C = (c.num_taps + kB - 2) / kB;
            const long long blocks = (c.num_samples + kB - 1) / kB;
            b.tiles = static_cast<int>((blocks + kNB - 1) / kNB);
            b.item0 = items;
            items += b.tiles;
            cmax = std::max(cmax, b.C);
            const Geo g = geo_of(b.C, b.n);
            CUtensorMap xm, sm;
            err = encode_rows(&xm, c.x, 4, b.n / kB, 2 * kB, 32, static_cast<uint32_t>(g.rows));
            if (err == cudaSuccess) {
                err = encode_rows(&sm, c.x, 4, b.n / kB, 2 * kB, 2 * kB,
                                  static_cast<uint32_t>(g.srows));
            }
            if (err != cudaSuccess) {
                return err;
            }
            for (int t = 0; t < b.tiles; ++t) {
                cost.push_back(tc_tile_us(b.C));
            }
            tc.push_back(b);
            xmaps.push_back(xm);
            smaps.push_back(sm);
        } else {
            PlainCapDev q{};
            q.x = static_cast<const float2*>(c.x);
            q.y = static_cast<float2*>(c.y);
            q.taps = c.taps;
            q.n = c.num_samples;
            q.num_taps = c.num_taps;
            q.tile0 = ptiles;
            const int tiles =
                static_cast<int>((c.num_samples + kPlainTileOutputs - 1) / kPlainTileOutputs);
            ptiles += tiles;
            for (int t = 0; t < tiles; ++t) {
                plain_cost.push_back(plain_tile_us(c.num_taps));
            }
            kmax_plain = std::max(kmax_plain, c.num_taps);
            pl.push_back(q);
        }
    }
    // The unit line: tensor-core items, window items (C = 1, 2, 3), plain tiles.
    int wbase[tcw::kCMax];
    int wunits[tcw::kCMax];
    int nwin = 0;
    for (int ci = 0; ci < tcw::kCMax; ++ci) {
        wbase[ci] = static_cast<int>(cost.size());
        wunits[ci] = static_cast<int>(wcost[ci].size());
        cost.insert(cost.end(), wcost[ci].begin(), wcost[ci].end());
        nwin += static_cast<int>(wc[ci].size());
    }
    const int pbase = static_cast<int>(cost.size());
    cost.insert(cost.end(), plain_cost.begin(), plain_cost.end());
    const int units = static_cast<int>(cost.size());
    auto* plan = new BatchPlan{};
    plan->tc_caps = static_cast<int>(tc.size()) + nwin;
    plan->plain_caps = static_cast<int>(pl.size());
    if (units == 0) {
        *out = plan;   // nothing to run
        return cudaSuccess;
    }
    // Shared memory: the tensor-core pipeline for the largest filter (the deepest scan ring,
    // then the most operand stages that fit), and up to three plain-tile regions.
    Layout lay{};
    int stages = 0;
    int sbufs = 0;
    if (!tc.empty()) {
        for (int sb = kScanBufsMax; sb >= 2 && stages == 0; sb -= 2) {
            for (int st : {6, 4, 2}) {
                if (batch_layout(cmax, st, sb).bytes <= kSmemMax) {
                    stages = st;
                    sbufs = sb;
                    lay = batch_layout(cmax, st, sb);
                    break;
                }
            }
        }
        if (stages == 0) {
            delete plan;
            return cudaErrorInvalidValue;
        }
    }
    // Plain tiles: three groups of two slots each where they fit (short filters), else as many
    // one-slot groups as fit.
    uint32_t region = 0;
    uint32_t slot = 0;
    int groups = 0;
    if (!pl.empty()) {
        slot = align_up(plain_layout(kmax_plain).bytes, 128);
        if (1024u + kPlainGroupsMax * 2u * slot <= kSmemMax) {
            region = 2u * slot;
            groups = kPlainGroupsMax;
        } else {
            region = slot;
            groups = std::min<int>(kPlainGroupsMax, static_cast<int>((kSmemMax - 1024u) / slot));
        }
        if (groups < 1) {
            delete plan;
            return cudaErrorInvalidValue;
        }
    }
    plan->stages = stages == 0 ? 2 : stages;
    plan->smem = std::max({tc.empty() ? 0u : lay.bytes, 1024u + groups * region, 120u * 1024u});
    // The window pipeline's layout (win_stages stages, win_strips strip slots) and its control
    // block in the last kilobyte.
    for (int ci = 0; ci < tcw::kCMax; ++ci) {
        if (!wc[ci].empty()) {
            const int C = ci + 1;
            plan->smem = std::max(
                plan->smem, tcw::win_layout(C, win_stages(C), win_strips(C), 4).bytes + 1024u);
        }
    }
    if (plan->smem > kSmemMax) {
        delete plan;
        return cudaErrorInvalidValue;
    }

    // Partition: the units on one line (tensor-core items, then plain tiles), cut into grid
    // contiguous pieces of about equal cost; blocks of the first pieces run tensor-core items
    // while the last ones run plain tiles, so tensor-bound and memory-bound work overlap.
    const int grid = std::min({sms, kBatchCtas, units});
    std::vector<double> prefix(units + 1, 0.0);
    for (int u = 0; u < units; ++u) {
        prefix[u + 1] = prefix[u] + cost[u];
    }
    std::vector<int> cta_item(grid + 1), cta_plain(grid + 1);
    std::vector<int> cta_win[tcw::kCMax];
    for (auto& cw : cta_win) {
        cw.assign(grid + 1, 0);
    }
    for (int b = 0; b <= grid; ++b) {
        int u = b == grid ? units
                          : static_cast<int>(std::lower_bound(prefix.begin(), prefix.end(),
                                                              prefix[units] * b / grid) -
                                             prefix.begin());
        u = std::min(u, units);
        cta_item[b] = std::min(u, items);
        for (int ci = 0; ci < tcw::kCMax; ++ci) {
            cta_win[ci][b] = std::min(std::max(u - wbase[ci], 0), wunits[ci]);
        }
        cta_plain[b] = std::max(u - pbase, 0);
    }
    for (int b = 1; b <= grid; ++b) {   // monotone after rounding
        cta_item[b] = std::max(cta_item[b], cta_item[b - 1]);
        for (int ci = 0; ci < tcw::kCMax; ++ci) {
            cta_win[ci][b] = std::max(cta_win[ci][b], cta_win[ci][b - 1]);
        }
        cta_plain[b] = std::max(cta_plain[b], cta_plain[b - 1]);
    }

    // One device buffer: capture table, tensor maps (128-byte aligned), block ranges, plain
    // captures.
    const uint32_t n_tc = static_cast<uint32_t>(tc.size());
    const uint32_t off_cap = 0;
    const uint32_t off_xmap = align_up(off_cap + n_tc * sizeof(BatchCap), 128);
    const uint32_t off_smap = off_xmap + n_tc * sizeof(CUtensorMap);
    const uint32_t off_item = align_up(off_smap + n_tc * sizeof(CUtensorMap), 16);
    const uint32_t off_plain = align_up(off_item + (grid + 1) * sizeof(int), 16);
    const uint32_t off_pcap = align_up(off_plain + (grid + 1) * sizeof(int), 16);
    uint32_t off_w = align_up(off_pcap + pl.size() * sizeof(PlainCapDev), 128);
    uint32_t off_wmap[tcw::kCMax], off_wcap[tcw::kCMax], off_wcta[tcw::kCMax];
    for (int ci = 0; ci < tcw::kCMax; ++ci) {
        off_wmap[ci] = off_w;
        off_wcap[ci] = align_up(off_wmap[ci] + wm[ci].size() * sizeof(CUtensorMap), 16);
        off_wcta[ci] = align_up(off_wcap[ci] + wc[ci].size() * sizeof(tcw::WinCapture), 16);
        off_w = align_up(off_wcta[ci] + (grid + 1) * sizeof(int), 128);
    }
    const uint32_t bytes = off_w;
    std::vector<unsigned char> host(bytes, 0);
    std::memcpy(host.data() + off_cap, tc.data(), n_tc * sizeof(BatchCap));
    std::memcpy(host.data() + off_xmap, xmaps.data(), n_tc * sizeof(CUtensorMap));
    std::memcpy(host.data() + off_smap, smaps.data(), n_tc * sizeof(CUtensorMap));
    std::memcpy(host.data() + off_item, cta_item.data(), (grid + 1) * sizeof(int));
    std::memcpy(host.data() + off_plain, cta_plain.data(), (grid + 1) * sizeof(int));
    std::memcpy(host.data() + off_pcap, pl.data(), pl.size() * sizeof(PlainCapDev));
    for (int ci = 0; ci < tcw::kCMax; ++ci) {
        std::memcpy(host.data() + off_wmap[ci], wm[ci].data(), wm[ci].size() * sizeof(CUtensorMap));
        std::memcpy(host.data() + off_wcap[ci], wc[ci].data(),
                    wc[ci].size() * sizeof(tcw::WinCapture));
        std::memcpy(host.data() + off_wcta[ci], cta_win[ci].data(), (grid + 1) * sizeof(int));
    }
    unsigned char* dev = nullptr;
    if ((err = cudaMalloc(&dev, bytes)) != cudaSuccess ||
        (err = cudaMemcpy(dev, host.data(), bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
        cudaFree(dev);
        delete plan;
        return err;
    }
    plan->dev = dev;
    plan->grid = grid;
    BatchView& v = plan->view;
    v.cap = reinterpret_cast<const BatchCap*>(dev + off_cap);
    v.xmap = reinterpret_cast<const CUtensorMap*>(dev + off_xmap);
    v.smap = reinterpret_cast<const CUtensorMap*>(dev + off_smap);
    v.cta_item = reinterpret_cast<const int*>(dev + off_item);
    v.cta_plain = reinterpret_cast<const int*>(dev + off_plain);
    v.pcap = reinterpret_cast<const PlainCapDev*>(dev + off_pcap);
    v.count = static_cast<int>(n_tc);
    v.pcount = static_cast<int>(pl.size());
    v.cmax = cmax;
    v.sbufs = sbufs == 0 ? 2 : sbufs;
    v.plain_groups = groups;
    v.plain_region = region;
    v.plain_slot = slot;
    v.maps_global = 1;
    for (int ci = 0; ci < tcw::kCMax; ++ci) {
        v.wcap[ci] = reinterpret_cast<const tcw::WinCapture*>(dev + off_wcap[ci]);
        v.wmap[ci] = reinterpret_cast<const CUtensorMap*>(dev + off_wmap[ci]);
        v.cta_win[ci] = reinterpret_cast<const int*>(dev + off_wcta[ci]);
        v.wcount[ci] = static_cast<int>(wc[ci].size());
    }
    v.win_ctl = plan->smem - 1024u;
    const void* fn = plan->stages == 6   ? reinterpret_cast<const void*>(fir_batch_list_kernel<6>)
                     : plan->stages == 4 ? reinterpret_cast<const void*>(fir_batch_list_kernel<4>)
                                         : reinterpret_cast<const void*>(fir_batch_list_kernel<2>);
    if ((err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(plan->smem))) != cudaSuccess) {
        fir_batch_plan_free(plan);
        return err;
    }
    *out = plan;
    return cudaSuccess;
}

cudaError_t fir_batch_plan_run(const BatchPlan* plan, cudaStream_t stream)
{
    if (plan->grid == 0) {
        return cudaSuccess;
    }
    const dim3 grid(static_cast<unsigned>(plan->grid));
    switch (plan->stages) {
    case 6:
        fir_batch_list_kernel<6><<<grid, kThreads, plan->smem, stream>>>(plan->view);
        break;
    case 4:
        fir_batch_list_kernel<4><<<grid, kThreads, plan->smem, stream>>>(plan->view);
        break;
    default:
        fir_batch_list_kernel<2><<<grid, kThreads, plan->smem, stream>>>(plan->view);
        break;
    }
    return cudaGetLastError();
}

cudaError_t fir_batch_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_batch, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_batch, &zero, sizeof(unsigned int));
}

}  // namespace rfx
