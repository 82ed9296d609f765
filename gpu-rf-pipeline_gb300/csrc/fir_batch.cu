// Batched tensor-core FIR: many captures, each with its own taps and length, in ONE persistent
// launch. No counterpart in the project, which runs such a batch as one launch per capture.
//
// Work list: every capture is cut into tiles of 96 blocks of 128 outputs (as fir_tc.cu); the
// (capture, tile) items are numbered capture by capture, and each block of the grid takes one
// contiguous range of items, the ranges chosen on the host so that every block gets about the
// same work (measured: about the same per tile whatever the filter). The capture table travels in the kernel parameters (48 bytes per
// capture), so a launch allocates nothing and can be captured in a CUDA graph.
//
// The per-tile pipeline is the one of fir_tc.cu (worker warps convert scaled FP16 hi/lo sample
// planes; h_hi x_hi goes to accumulator H in groups of at most 18 MMAs, each drained into FP32
// running sums in registers, the cross products to accumulator X, drained once per tile; one
// thread issues the MMAs from a lean loop), with two differences: samples are loaded from global
// memory by the workers (one tensor map per capture would not fit the parameter space), and when
// a block's range moves on to the next capture its tap strip is rebuilt — after every MMA of the
// previous capture has completed, which the drain of its last tile's X accumulator guarantees.
#include "fir_tc.cuh"
#include "fir_plain.cuh"
#include "tc_common.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace rfx {

static __device__ unsigned int g_fault_fir_batch;

namespace {

using namespace tc;

constexpr int kB = 128;
constexpr int kNB = 96;
constexpr int kN = 2 * kNB;
constexpr int kStagesPerTile = kB / 16;
constexpr int kWorkerWarps = 16;
constexpr int kWorkers = kWorkerWarps * 32;
constexpr int kMmaWarp = 16;
constexpr int kThreads = 17 * 32;
constexpr int kCols = kN / 4;
constexpr int kHGroup = 18;       // MMAs per H accumulation, at most
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kXCol = kN;
constexpr uint32_t kIdesc = idesc_f16(kB, kN);
constexpr int kBatchCaps = 192;   // captures per launch
constexpr int kBatchCtas = 192;   // blocks per launch (one per SM)

struct BatchCap {
    const float2* x;
    float2* y;
    const float* taps;
    long long n;
    int num_taps;
    int C;
    int tiles;
    int item0;   // first item of this capture in the work list
};

struct BatchParams {
    BatchCap cap[kBatchCaps];
    int count;
    int cmax;
    int cta_item[kBatchCtas + 1];
};

struct Layout {
    int rows_max;
    uint32_t pitch, split, stage;
    int tcount_max;
    uint32_t taps_hi, taps_lo, stages0, bytes;
};

__host__ __device__ inline Layout batch_layout(int cmax, int stages)
{
    Layout l;
    l.rows_max = kNB + cmax;
    l.pitch = static_cast<uint32_t>(2 * l.rows_max) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    l.tcount_max = 16 * cmax + 31;
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount_max);
    l.stages0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount_max) + 127u) & ~127u;
    l.bytes = l.stages0 + l.stage * static_cast<uint32_t>(stages);
    return l;
}

struct Ctrl {
    unsigned long long full[8];
    unsigned long long empty[8];
    unsigned long long pfull;
    unsigned long long pempty;
    unsigned long long xfull;
    unsigned long long xempty;
    unsigned long long reduce[2];
    unsigned long long tap_reduce[2];
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t warp_max[2][kWorkerWarps];
    uint32_t tap_max[2][kWorkerWarps];
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// Capture of a work-list item, searched forward from a cursor (items only increase).
__device__ __forceinline__ int capture_of(const BatchParams& p, int item, int cursor)
{
    while (cursor + 1 < p.count && p.cap[cursor + 1].item0 <= item) {
        ++cursor;
    }
    return cursor;
}

// H groups of a tile of a capture with P chunks: `ksg` whole K-steps (P <= 18), or `gpk`
// groups of at most `cpg` chunks per K-step (P > 18); see fir_tc.cu.
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

// Last K-step of group gi.
__device__ __forceinline__ int h_group_last_step(const HGroups& g, int gi)
{
    return g.gpk == 1 ? min(kStagesPerTile, (gi + 1) * g.ksg) - 1 : gi / g.gpk;
}

}  // namespace

template <int S>
__global__ void __launch_bounds__(kThreads, 1) fir_batch_kernel(const __grid_constant__ BatchParams p)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const Layout lay = batch_layout(p.cmax, S);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_batch;
    const int first_item = p.cta_item[blockIdx.x];
    const int my_items = p.cta_item[blockIdx.x + 1] - first_item;
    const int my_steps = my_items * kStagesPerTile;
    if (my_items <= 0) {
        return;  // uniform for the whole block: nothing allocated yet
    }

    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kWorkerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.reduce[i]), kWorkerWarps);
            mbar_init(smem_u32(&ctl.tap_reduce[i]), kWorkerWarps);
        }
        mbar_init(smem_u32(&ctl.pfull), 1);
        mbar_init(smem_u32(&ctl.pempty), kWorkerWarps);
        mbar_init(smem_u32(&ctl.xfull), 1);
        mbar_init(smem_u32(&ctl.xempty), kWorkerWarps);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp < kWorkerWarps) {
        const int quarter = warp & 3;
        const int slice = warp >> 2;
        const int r = kB - 1 - (quarter * 32 + lane);
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(slice * kCols);
        const int wtid = threadIdx.x;
        int ex_even = 0;     // scale exponents of even and odd items
        int ex_odd = 0;
        int eh = 0;          // tap scale of the strip currently in shared memory
        int switches = 0;    // tap-strip rebuilds so far (phase of tap_reduce)
        int cur_prod = capture_of(p, first_item, 0);
        int cur_drain = cur_prod;
        int cur_scan = cur_prod;

        auto item_capture = [&](int local_item, int& cursor) -> int {
            cursor = capture_of(p, first_item + local_item, cursor);
            return cursor;
        };
        auto window = [&](const BatchCap& c, int tile, long long& lo_s, long long& hi_s) {
            const long long j0 = static_cast<long long>(tile) * kNB;
            const long long win0 = (j0 - c.C) * kB;
            lo_s = win0 > 0 ? win0 : 0;
            hi_s = (j0 + kNB) * kB < c.n ? (j0 + kNB) * kB : c.n;
        };
        auto load_pair = [&](const float2* x, long long s, long long hi_s) -> uint32_t {
            if (s + 1 < hi_s) {
                return absmax4(__ldg(reinterpret_cast<const float4*>(x + s)));
            }
            if (s < hi_s) {
                const float2 w2 = __ldg(x + s);
                return max(absbits(w2.x), absbits(w2.y));
            }
            return 0u;
        };
        auto reduce_scale = [&](int k, uint32_t m) -> bool {
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            const int rb = k & 1;
            if (lane == 0) {
                ctl.warp_max[rb][warp] = m;
                mbar_arrive(smem_u32(&ctl.reduce[rb]));
            }
            if (!mbar_wait_bounded(smem_u32(&ctl.reduce[rb]), (k >> 1) & 1, fault,
                                   kFaultStageEmpty, abort)) {
                return false;
            }
            uint32_t tmax = 0;
#pragma unroll
            for (int w = 0; w < kWorkerWarps; ++w) {
                tmax = max(tmax, ctl.warp_max[rb][w]);
            }
            if (k & 1) {
                ex_odd = scale_exponent(tmax);
            } else {
                ex_even = scale_exponent(tmax);
            }
            return true;
        };
        // The tap strip of capture c (every worker writes its share after its own drain of the
        // last partial sum that used the old strip).
        auto build_strip = [&](const BatchCap& c) -> bool {
            uint32_t m = 0;
            for (int k = wtid; k < c.num_taps; k += kWorkers) {
                m = max(m, absbits(__ldg(c.taps + k)));
            }
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            const int rb = switches & 1;
            if (lane == 0) {
                ctl.tap_max[rb][warp] = m;
                mbar_arrive(smem_u32(&ctl.tap_reduce[rb]));
            }
            if (!mbar_wait_bounded(smem_u32(&ctl.tap_reduce[rb]), (switches >> 1) & 1, fault,
                                   kFaultStageEmpty, abort)) {
                return false;
            }
            uint32_t tmax = 0;
#pragma unroll
            for (int w = 0; w < kWorkerWarps; ++w) {
                tmax = max(tmax, ctl.tap_max[rb][w]);
            }
            ++switches;
            eh = scale_exponent(tmax);
            const float fa = exp2i(eh / 2);
            const float fb = exp2i(eh - eh / 2);
            const int dmax = (c.C + 1) * kB - 1;
            const int pairs = (16 * c.C + 31) * 32;
            for (int i = wtid; i < pairs; i += kWorkers) {
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
            return true;  // made visible to the MMAs by the fence before the next full arrive
        };
        uint32_t next_max = 0;
        auto produce = [&](int v) -> bool {
            const int k = v / kStagesPerTile;
            const int st = v % kStagesPerTile;
            const int ci = item_capture(k, cur_prod);
            const BatchCap& c = p.cap[ci];
            const int tile = first_item + k - c.item0;
            const long long j0 = static_cast<long long>(tile) * kNB;
            uint32_t pre[3] = {0u, 0u, 0u};
            const bool has_next = k + 1 < my_items;
            if (has_next) {
                const int cn = item_capture(k + 1, cur_scan);
                const BatchCap& c2 = p.cap[cn];
                long long lo_n, hi_n;
                window(c2, first_item + k + 1 - c2.item0, lo_n, hi_n);
                const long long pairs = (hi_n - lo_n + 1) / 2;
                const long long per = (pairs + kStagesPerTile - 1) / kStagesPerTile;
                const long long end = (st + 1) * per < pairs ? (st + 1) * per : pairs;
                long long idx = st * per + wtid;
#pragma unroll
                for (int i = 0; i < 3; ++i, idx += kWorkers) {
                    if (idx < end) {
                        pre[i] = load_pair(c2.x, lo_n + 2 * idx, hi_n);
                    }
                }
                for (; idx < end; idx += kWorkers) {
                    pre[0] = max(pre[0], load_pair(c2.x, lo_n + 2 * idx, hi_n));
                }
            }
            const int ex = (k & 1) ? ex_odd : ex_even;
            const float fa = exp2i(ex / 2);
            const float fb = exp2i(ex - ex / 2);
            const int slot = v % S;
            if (!mbar_wait_bounded(smem_u32(&ctl.empty[slot]), ((v / S) & 1) ^ 1, fault,
                                   kFaultStageEmpty, abort)) {
                return false;
            }
            const uint32_t stage = sbase + lay.stages0 + static_cast<uint32_t>(slot) * lay.stage;
            const int items = (kNB + c.C) * 8;
            for (int f = wtid; f < items; f += kWorkers) {
                const int b = f >> 3;
                const int q = f & 7;
                const long long sidx = (j0 - c.C + b) * kB + 16 * st + 2 * q;
                float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (sidx >= 0 && sidx + 1 < c.n) {
                    v4 = __ldg(reinterpret_cast<const float4*>(c.x + sidx));
                } else if (sidx >= 0 && sidx < c.n) {
                    const float2 w2 = __ldg(c.x + sidx);
                    v4.x = w2.x;
                    v4.y = w2.y;
                }
                uint32_t re_hi, re_lo, im_hi, im_lo;
                split2(v4.x * fa * fb, v4.z * fa * fb, re_hi, re_lo);
                split2(v4.y * fa * fb, v4.w * fa * fb, im_hi, im_lo);
                const uint32_t plane = static_cast<uint32_t>(q >> 2) * lay.pitch;
                const uint32_t elem = static_cast<uint32_t>(q & 3) * 4u;
                const uint32_t row_re = plane + static_cast<uint32_t>(2 * b) * 16u + elem;
                sts32(stage + row_re, re_hi);
                sts32(stage + row_re + 16u, im_hi);
                sts32(stage + lay.split + row_re, re_lo);
                sts32(stage + lay.split + row_re + 16u, im_lo);
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.full[slot]));
            }
            if (has_next) {
                next_max = max(next_max, max(pre[0], max(pre[1], pre[2])));
                if (st == kStagesPerTile - 1) {
                    if (!reduce_scale(k + 1, next_max)) {
                        return false;
                    }
                    next_max = 0;
                }
            }
            return true;
        };
        // A K-step that starts a new capture (not the block's first) needs a new tap strip.
        int sw_cursor = cur_prod;
        auto starts_capture = [&](int v) -> bool {
            if (v % kStagesPerTile != 0 || v == 0) {
                return false;
            }
            const int k = v / kStagesPerTile;
            const int a = item_capture(k - 1, sw_cursor);
            const int b = capture_of(p, first_item + k, a);
            return a != b;
        };

        bool ok = true;
        {
            // Prologue: tap strip and scale of the first item, then the first stages.
            const BatchCap& c0 = p.cap[cur_prod];
            ok = build_strip(c0);
            long long lo0, hi0;
            window(c0, first_item - c0.item0, lo0, hi0);
            uint32_t m = 0;
            const long long pairs = (hi0 - lo0 + 1) / 2;
            for (long long base = 0; base < pairs && ok; base += 8 * kWorkers) {
                uint32_t part[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const long long idx = base + wtid + i * kWorkers;
                    part[i] = idx < pairs ? load_pair(c0.x, lo0 + 2 * idx, hi0) : 0u;
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    m = max(m, part[i]);
                }
            }
            ok = ok && reduce_scale(0, m);
        }
        int produced = 0;
        while (ok && produced < S && produced < my_steps && !starts_capture(produced)) {
            ok = produce(produced++);
        }
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
        int g = 0;   // H groups drained so far (the pfull / pempty phase)
        int gi = 0;  // next group of the current item
        for (int u = 0; u < my_steps && ok && !*abort; ++u) {
            const int k = u / kStagesPerTile;
            const int st = u % kStagesPerTile;
            const int ci = item_capture(k, cur_drain);
            const BatchCap& c = p.cap[ci];
            const HGroups grp = h_groups(c.C + 1, S);
            while (gi < grp.per_tile && h_group_last_step(grp, gi) <= st) {
                if (!mbar_wait_bounded(smem_u32(&ctl.pfull), g & 1, fault, kFaultAccumFull,
                                       abort)) {
                    ok = false;
                    break;
                }
                drain(0);
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.pempty));
                }
                ++g;
                ++gi;
            }
            if (!ok) {
                break;
            }
            if (st == kStagesPerTile - 1) {
                if (!mbar_wait_bounded(smem_u32(&ctl.xfull), k & 1, fault, kFaultAccumFull,
                                       abort)) {
                    break;
                }
                drain(kXCol);
                if (lane == 0) {
                    mbar_arrive(smem_u32(&ctl.xempty));
                }
                const int shift = -(((k & 1) ? ex_odd : ex_even) + eh);
                const float fa = exp2i(shift / 2);
                const float fb = exp2i(shift - shift / 2);
                const long long jb0 =
                    static_cast<long long>(first_item + k - c.item0) * kNB + slice * (kCols / 2);
#pragma unroll
                for (int b = 0; b < kCols / 2; ++b) {
                    const long long o = (jb0 + b) * kB + r;
                    if (o < c.n) {
                        c.y[o] = make_float2(acc[2 * b] * fa * fb, acc[2 * b + 1] * fa * fb);
                    }
                    acc[2 * b] = 0.0f;
                    acc[2 * b + 1] = 0.0f;
                }
                gi = 0;
            }
            while (ok && produced < my_steps && produced <= u + S) {
                if (starts_capture(produced)) {
                    if (produced != u + 1) {
                        break;  // wait until every MMA of the old capture has been drained
                    }
                    ok = build_strip(p.cap[capture_of(p, first_item + produced / kStagesPerTile,
                                                      cur_prod)]);
                    if (!ok) {
                        break;
                    }
                }
                ok = produce(produced++);
            }
        }
    } else if (lane == 0) {
        // MMA issuer: lean loop, per MMA one descriptor step and the MMA (see fir_tc.cu).
        const uint32_t taps_hi = sbase + lay.taps_hi;
        const uint32_t taps_lo = sbase + lay.taps_lo;
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        const uint32_t stages_units = (sbase + lay.stages0) >> 4;
        const uint32_t h_acc = tmem;
        const uint32_t x_acc = tmem + kXCol;
        int cursor = capture_of(p, first_item, 0);
        int g = 0;
        int ready = 0;
        bool stop = false;
        for (int k = 0; k < my_items && !stop && !*abort; ++k) {
            cursor = capture_of(p, first_item + k, cursor);
            const int C = p.cap[cursor].C;
            const int P = C + 1;
            const HGroups grp = h_groups(P, S);
            const uint32_t a_hi0 = (taps_hi >> 4) + static_cast<uint32_t>(16 * C) * 8u;
            const uint32_t a_lo0 = (taps_lo >> 4) + static_cast<uint32_t>(16 * C) * 8u;
            const uint32_t b_base = stages_units + static_cast<uint32_t>(2 * C);
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
                    uint32_t a = a_hi0 + static_cast<uint32_t>(2 * st - 16 * c0) * 8u;
                    uint32_t b = b_base + static_cast<uint32_t>(slot) * stage_units -
                                 static_cast<uint32_t>(2 * c0);
                    for (int c = c0; c < c1; ++c) {
                        mma_f16<kIdesc>(h_acc, a_desc | a, b_desc | b, acc);
                        acc = 1;
                        a -= 128;
                        b -= 2;
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
                    uint32_t ah = a_hi0 + off;
                    uint32_t al = a_lo0 + off;
                    uint32_t b = b_base + static_cast<uint32_t>(slot) * stage_units -
                                 static_cast<uint32_t>(2 * c0);
                    for (int c = c0; c < c1; ++c) {
                        mma_f16<kIdesc>(x_acc, a_desc | ah, b_desc | (b + split_units), acc);
                        mma_f16<kIdesc>(x_acc, a_desc | al, b_desc | b, 1u);
                        acc = 1;
                        ah -= 128;
                        al -= 128;
                        b -= 2;
                    }
                    if (c1 == P) {
                        mma_commit(smem_u32(&ctl.empty[slot]));
                    }
                }
            }
            if (!stop) {
                mma_commit(smem_u32(&ctl.xfull));
            }
        }
        mma_commit(smem_u32(&ctl.teardown));
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    }

    fence_before();
    __syncthreads();
    fence_after();
    if (warp == kMmaWarp) {
        tmem_dealloc(tmem, kTmemCols);
    }
}

namespace {

// Splits the items of `caps` into `parts` contiguous ranges of about equal cost (every range
// non-empty; parts <= total_items).
void partition(const std::vector<BatchCap>& caps, int total_items, int parts, int* cta_item)
{
    std::vector<double> prefix(total_items + 1, 0.0);
    for (const BatchCap& c : caps) {
        // Measured on GB300: a tile costs about the same whatever its filter (the workers'
        // conversion of its window bounds it), 5 % more at 9 chunks than at 2.
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
cudaError_t launch_batch(const BatchParams& params, int grid, int cmax, cudaStream_t stream)
{
    const Layout lay = batch_layout(cmax, S);
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
    return fir_tc_supported(num_taps) && batch_layout((num_taps + kB - 2) / kB, 2).bytes <= 227u * 1024u;
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
        caps.push_back(b);
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
        }
        params->count = static_cast<int>(chunk);
        params->cmax = cmax;
        partition(part, items, grid, params->cta_item);
        if (batch_layout(cmax, 4).bytes <= 227u * 1024u) {
            err = launch_batch<4>(*params, grid, cmax, stream);
        } else {
            err = launch_batch<2>(*params, grid, cmax, stream);
        }
        delete params;
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
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
