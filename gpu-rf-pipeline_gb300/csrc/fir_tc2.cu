// Tensor-core FIR on CTA pairs (2-SM tcgen05 MMAs, M = 256) for sm_103a, split FP16.
//
//   y[n] = sum_{k<K} h[k] x[n-k],  x[m < 0] = 0                              (src/fir.cu:1-5)
//
// The same block-Toeplitz GEMM as the single-CTA form (fir_tc.cu), with blocks of B = 256
// outputs so that one MMA covers M = 256 output rows across a pair of CTAs: per MMA each SM
// reads half of A and half of B from its own shared memory, which halves the operand traffic
// per SM (a single-CTA M = 128, N = 192 MMA needs 107 of the SM's 128 shared-memory bytes per
// clock at full rate; this form needs 75).
//
// With X[s][j] = x[jB + s] the output block j is Y[:, j] = sum_{c=0}^{C} T_c X[:, j - c],
// T_c(r, s) = h[cB + r - s], C = floor((K + B - 2) / B). A tile is 96 consecutive blocks
// (24576 outputs); MMA N = 192 (column 2 j' + {0: I, 1: Q}); CTA r of the pair supplies the
// columns of blocks 48 r .. 48 r + 47, converting its own window of 48 + C input blocks.
//
//  * A: output rows are stored reversed (MMA row i holds output 255 - i), so an 8 x 8 core
//    matrix of A depends only on (row group + K group): every T_c lives in one strip of core
//    matrices G[t][q][e] = h[(C+1)B - 1 - 8t - q - e]; a K-step's A is a descriptor into the
//    strip with leading- and stride-byte offsets 128 (overlapping reads). CTA r holds MMA rows
//    128 r .. +127, i.e. the strip from core matrix 16 r on, at the same shared offset.
//  * B: per K-step two 8-sample planes with one 16-byte row per (window block, component) at a
//    16-byte pitch; the shift by c blocks is a start address 32 c bytes further.
//
// Split precision, accumulation and roles as in the single-CTA form: x' = 2^ex x (ex per tile,
// common to the pair: each CTA scans its window and the two maxima are exchanged through
// distributed shared memory) and h' = 2^eh h split into FP16 hi + lo; h_hi x_hi goes to
// accumulator H in groups of at most 18 MMAs, each group added into FP32 running sums in
// registers (the tensor core rounds toward zero); the cross products go to accumulator X, drained
// once per tile. Roles per CTA: warps 0-15 drain (running sums, outputs), warps 16-21 produce (scan,
// convert), warp 22 issues the copies, warp 23 issues the MMAs for the pair (even CTA) or
// forwards the odd CTA's hand-offs (stage full, accumulators drained) as one cross-CTA arrive
// each on the even CTA's mbarriers; the MMA commits arrive on both CTAs' mbarriers
// (multicast). Every wait is bounded in time.
#include "fir_tc2.cuh"
#include "tc_common.cuh"
#include "tc_pair.cuh"
#include "tmap.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_fir_tc2;

namespace {

using namespace tc;
using namespace pair;

constexpr int kB = 256;                  // outputs per block = MMA M (pair)
constexpr int kRowsPerCta = 128;         // MMA rows per CTA
constexpr int kNB = 96;                  // blocks per tile (pair)
constexpr int kNBc = kNB / 2;            // blocks per CTA
constexpr int kN = 2 * kNB;              // MMA N
constexpr int kStepsPerTile = kB / 16;   // K-steps of 16 samples
constexpr int kStepsPerStage = 2;        // an operand stage holds 32 samples of each block
constexpr int kStagesPerTile = kStepsPerTile / kStepsPerStage;
constexpr int kDrainWarps = 16;          // hold the running sums, drain, store
constexpr int kProducerWarps = 6;        // scan, convert
constexpr int kProducers = kProducerWarps * 32;
constexpr int kFirstProducerWarp = kDrainWarps;
constexpr int kTmaWarp = kDrainWarps + kProducerWarps;
constexpr int kMmaWarp = kTmaWarp + 1;
constexpr int kThreads = (kMmaWarp + 1) * 32;
constexpr int kCols = kN / 4;            // running sums per worker thread
constexpr int kHGroup = 18;              // MMAs per H accumulation, at most
constexpr int kRaw = 3;                  // TMA raw-sample ring depth
constexpr int kScanBufsMax = 4;          // scan slice ring depth (slices copied depth-2 ahead)
constexpr int kMaxStages = 8;
constexpr uint32_t kTmemCols = 512;      // H (kN columns) and X (kN columns)
constexpr uint32_t kXCol = kN;
constexpr uint32_t kIdesc = idesc_f16(kB, kN);

struct Layout {
    int C;               // previous blocks a block reaches back to
    int rows;            // window blocks per CTA and tile: kNBc + C
    int srows;           // 128-sample rows per scan slice: ceil(2 rows / 8)
    uint32_t pitch;      // bytes per plane (2 rows * 16 B per block + 16)
    uint32_t split;      // bytes of one split (hi or lo) of a stage: 4 planes
    uint32_t stage;      // bytes per operand stage: hi + lo
    uint32_t raw;        // bytes per raw stage: rows * 32 samples * 8 B
    uint32_t scan;       // bytes per scan slice: srows * 128 samples * 8 B
    int tcount;          // core matrices of this CTA's tap strip
    int sbufs;           // scan slice buffers
    uint32_t taps_hi, taps_lo, raw0, scan0, stages0, bytes;
};

__host__ __device__ inline Layout tc2_layout(int num_taps, int stages, int sbufs)
{
    Layout l;
    l.C = (num_taps + kB - 2) / kB;
    l.rows = kNBc + l.C;
    l.srows = (2 * l.rows + kStagesPerTile - 1) / kStagesPerTile;
    l.pitch = static_cast<uint32_t>(2 * l.rows) * 16u + 16u;
    l.split = 4u * l.pitch;
    l.stage = 2u * l.split;
    l.raw = static_cast<uint32_t>(l.rows) * 256u;
    l.scan = static_cast<uint32_t>(l.srows) * 1024u;
    l.tcount = 32 * l.C + 47;
    l.sbufs = sbufs;
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount);
    l.raw0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount) + 127u) & ~127u;
    l.scan0 = l.raw0 + kRaw * l.raw;
    l.stages0 = l.scan0 + static_cast<uint32_t>(sbufs) * l.scan;
    l.bytes = l.stages0 + l.stage * static_cast<uint32_t>(stages);
    return l;
}

// Control block at the start of shared memory (same offsets in both CTAs).
struct Ctrl {
    unsigned long long full[kMaxStages];      // even CTA: producer-warp arrivals of both CTAs
    unsigned long long empty[kMaxStages];     // both: MMA commit
    unsigned long long raw_full[kRaw];
    unsigned long long raw_empty[kRaw];
    unsigned long long scan_full[kScanBufsMax];
    unsigned long long scan_empty[kScanBufsMax];
    unsigned long long pfull;                 // both: H group summed
    unsigned long long pempty;                // even CTA: H drained by both
    unsigned long long xfull;                 // both: X of a tile summed
    unsigned long long xempty;                // even CTA: X drained by both
    unsigned long long sready[4];             // this CTA: the scale of tile k is in ex[k % 4]
    unsigned long long xchg[2];               // the other CTA's maximum has arrived
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t pmax[2][kProducerWarps];
    int ex[4];
    uint32_t peer_max[2];                     // written by the other CTA
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// H groups of a tile: `ksg` whole K-steps (P <= 18 chunks; fewer K-steps than operand stages,
// since a group holds its stages until its X MMAs), or `gpk` groups of at most `cpg` chunks
// per K-step (P > 18).
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
        g.ksg = max(1, min(kHGroup / P, kStepsPerStage * (S - 1)));
        g.gpk = 1;
        g.cpg = P;
        g.per_tile = (kStepsPerTile + g.ksg - 1) / g.ksg;
    } else {
        g.ksg = 1;
        g.gpk = (P + kHGroup - 1) / kHGroup;
        g.cpg = (P + g.gpk - 1) / g.gpk;
        g.gpk = (P + g.cpg - 1) / g.cpg;
        g.per_tile = kStepsPerTile * g.gpk;
    }
    return g;
}

__device__ __forceinline__ void h_group_range(const HGroups& g, int P, int gi, int& st0, int& st1,
                                              int& c0, int& c1)
{
    if (g.gpk == 1) {
        st0 = gi * g.ksg;
        st1 = min(kStepsPerTile, st0 + g.ksg);
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

// xmap: x as rows of 512 floats (one 256-sample block), boxes of 64 floats x `rows` (one
// stage's samples of a CTA window). smap: x as rows of 256 floats (128 samples), boxes of
// 256 floats x `srows` (a scan slice).
template <int S>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kThreads, 1)
fir_tc2_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap smap,
               const float2* __restrict__ x, const float* __restrict__ taps,
               float2* __restrict__ y, long long n, int num_taps, int num_tiles, int sbufs)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const Layout lay = tc2_layout(num_taps, S, sbufs);
    const int C = lay.C;
    const int P = C + 1;                       // chunks per K-step
    const HGroups grp = h_groups(P, S);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();      // 0: issues the MMAs
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_tc2;
    const int pair_id = static_cast<int>(blockIdx.x) >> 1;
    const int pairs = static_cast<int>(gridDim.x) >> 1;
    // This pair's tiles: pair_id, + pairs, ...; stages are numbered v = 8 k + s, each holding
    // K-steps 2 s and 2 s + 1 of tile k.
    const int my_tiles = pair_id < num_tiles ? (num_tiles - 1 - pair_id) / pairs + 1 : 0;
    const int my_steps = my_tiles * kStagesPerTile;
    const int scan_slices = my_tiles > 1 ? (my_tiles - 1) * kStagesPerTile : 0;
    const long long full_blocks = n / kB;      // rows of xmap
    const long long full_halves = n / (kB / 2);  // rows of smap
    auto tile_of = [&](int k) { return pair_id + k * pairs; };
    // First window block of this CTA for tile k.
    auto win0 = [&](int k) {
        return static_cast<long long>(tile_of(k)) * kNB + kNBc * static_cast<int>(rank) - C;
    };

    // ---- setup ------------------------------------------------------------------------------
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps + (rank == 0 ? 1 : 0));
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
        mbar_init(smem_u32(&ctl.pfull), 1);
        mbar_init(smem_u32(&ctl.pempty), kDrainWarps + (rank == 0 ? 1 : 0));
        mbar_init(smem_u32(&ctl.xfull), 1);
        mbar_init(smem_u32(&ctl.xempty), kDrainWarps + (rank == 0 ? 1 : 0));
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.xchg[i]), 1);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(smem_u32(&ctl.sready[i]), 1);
        }
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        ctl.tap_max = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc_pair(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    // Scan slice q: the next tile's (q / 8 + 1) window, 128-sample rows (q % 8) srows .. +srows.
    auto issue_scan = [&](int q) {
        const int kn = q / kStagesPerTile + 1;
        const uint32_t bar = smem_u32(&ctl.scan_full[q % sbufs]);
        mbar_arrive_expect_tx(bar, lay.scan);
        tma_load_2d(sbase + lay.scan0 + static_cast<uint32_t>(q % sbufs) * lay.scan, &smap, 0,
                    static_cast<int>(2 * win0(kn)) + (q % kStagesPerTile) * lay.srows, bar);
    };
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int u = 0; u < kRaw && u < my_steps; ++u) {
            const uint32_t bar = smem_u32(&ctl.raw_full[u]);
            mbar_arrive_expect_tx(bar, lay.raw);
            tma_load_2d(sbase + lay.raw0 + u * lay.raw, &xmap, 64 * (u % kStagesPerTile),
                        static_cast<int>(win0(u / kStagesPerTile)), bar);
        }
        for (int q = 0; q < sbufs - 2 && q < scan_slices; ++q) {
            issue_scan(q);
        }
    }
    // Largest tap magnitude, then this CTA's part of the tap strip (from core matrix 16 rank).
    {
        uint32_t m = 0;
        for (int k = threadIdx.x; k < num_taps; k += kThreads) {
            m = max(m, absbits(__ldg(taps + k)));
        }
        m = __reduce_max_sync(0xFFFFFFFFu, m);
        if (lane == 0) {
            atomicMax(&ctl.tap_max, m);
        }
    }
    __syncthreads();
    const int eh = scale_exponent(ctl.tap_max);
    {
        const float fa = exp2i(eh / 2);
        const float fb = exp2i(eh - eh / 2);
        const int dmax = (C + 1) * kB - 1 - 8 * 16 * static_cast<int>(rank);
        const int npairs = lay.tcount * 32;   // two adjacent elements per item
        for (int i = threadIdx.x; i < npairs; i += kThreads) {
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
    cluster_sync_all();   // both CTAs' barriers are initialized before any remote arrival
    fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp < kDrainWarps) {
        // ---- drain warps: running sums, outputs ----------------------------------------------
        const int quarter = warp & 3;
        const int slice = warp >> 2;                       // columns kCols * slice .. +kCols-1
        const int r = kB - 1 - kRowsPerCta * static_cast<int>(rank) - (quarter * 32 + lane);
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
        // Drained-accumulator hand-offs: local arrivals (the odd CTA's are forwarded to the
        // even CTA by warp 23).
        auto arrive_lead = [&](unsigned long long* local) {
            if (lane == 0) {
                mbar_arrive(smem_u32(local));
            }
        };
        bool ok = true;
        int g = 0;
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            for (int gi = 0; gi < grp.per_tile; ++gi, ++g) {
                if (!mbar_wait_cluster_bounded(smem_u32(&ctl.pfull), g & 1, fault, kFaultAccumFull,
                                       abort)) {
                    ok = false;
                    break;
                }
                drain(0);
                arrive_lead(&ctl.pempty);
            }
            if (!ok ||
                !mbar_wait_cluster_bounded(smem_u32(&ctl.xfull), k & 1, fault, kFaultAccumFull, abort)) {
                break;
            }
            drain(kXCol);
            arrive_lead(&ctl.xempty);
            // The tile's sample scale (common to the pair), published by this CTA's producers.
            if (!mbar_wait_bounded(smem_u32(&ctl.sready[k & 3]), (k >> 2) & 1, fault, kFaultScale,
                                   abort)) {
                break;
            }
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k & 3]);
            const int shift = -(ex + eh);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            // Row r of blocks 24 slice .. +23.
            const long long jb0 = static_cast<long long>(tile_of(k)) * kNB + slice * (kCols / 2);
#pragma unroll
            for (int b = 0; b < kCols / 2; ++b) {
                const long long o = (jb0 + b) * kB + r;
                if (o < n) {
                    y[o] = make_float2(acc[2 * b] * fa * fb, acc[2 * b + 1] * fa * fb);
                }
                acc[2 * b] = 0.0f;
                acc[2 * b + 1] = 0.0f;
            }
        }
    } else if (warp < kFirstProducerWarp + kProducerWarps) {
        // ---- producers: scales, operand stages -----------------------------------------------
        const int pw = warp - kFirstProducerWarp;
        const int ptid = static_cast<int>(threadIdx.x) - kFirstProducerWarp * 32;
        int ex_even = 0;
        int ex_odd = 0;
        uint32_t next_max = 0;

        auto load_pair = [&](long long s, long long hi_s) -> uint32_t {
            if (s + 1 < hi_s) {
                return absmax4(__ldg(reinterpret_cast<const float4*>(x + s)));
            }
            if (s < hi_s) {
                const float2 w2 = __ldg(x + s);
                return max(absbits(w2.x), absbits(w2.y));
            }
            return 0u;
        };
        // Tile k's scale: this CTA's producers' maxima, then the other CTA's; published to the
        // drain warps.
        auto reduce_scale = [&](int k, uint32_t m) -> bool {
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            const int rb = k & 1;
            if (lane == 0) {
                ctl.pmax[rb][pw] = m;
            }
            asm volatile("bar.sync 1, %0;" ::"n"(kProducers) : "memory");
            uint32_t tmax = 0;
#pragma unroll
            for (int w = 0; w < kProducerWarps; ++w) {
                tmax = max(tmax, ctl.pmax[rb][w]);
            }
            if (ptid == 0) {
                st_cluster_u32(cluster_map(smem_u32(&ctl.peer_max[rb]), rank ^ 1u), tmax);
                mbar_arrive_cluster(cluster_map(smem_u32(&ctl.xchg[rb]), rank ^ 1u));
            }
            if (!mbar_wait_cluster_bounded(smem_u32(&ctl.xchg[rb]), (k >> 1) & 1, fault, kFaultScale,
                                   abort)) {
                return false;
            }
            tmax = max(tmax, *reinterpret_cast<volatile uint32_t*>(&ctl.peer_max[rb]));
            const int ex = scale_exponent(tmax);
            if (k & 1) {
                ex_odd = ex;
            } else {
                ex_even = ex;
            }
            if (ptid == 0) {
                ctl.ex[k & 3] = ex;
                mbar_arrive(smem_u32(&ctl.sready[k & 3]));
            }
            return true;
        };
        // Scan slice q: rows past the window are ignored; the partial last 128-sample row lies
        // outside smap (the copy reads zeros there) and is read from global memory.
        auto consume_slice = [&](int q) -> bool {
            const int qb = q % sbufs;
            if (!mbar_wait_bounded(smem_u32(&ctl.scan_full[qb]), (q / sbufs) & 1, fault,
                                   kFaultTileLoad, abort)) {
                return false;
            }
            const int k = q / kStagesPerTile + 1;
            const int r0 = (q % kStagesPerTile) * lay.srows;
            const uint32_t buf = sbase + lay.scan0 + static_cast<uint32_t>(qb) * lay.scan;
            const int quads = min(lay.srows, 2 * lay.rows - r0) * 64;
            uint32_t m = next_max;
            for (int f = ptid; f < quads; f += kProducers) {
                m = max(m, absmax4(lds128(buf + static_cast<uint32_t>(f) * 16u)));
            }
            const long long tail_row = full_halves - 2 * win0(k) - r0;
            if (tail_row >= 0 && tail_row * 64 < quads && ptid < 64) {
                m = max(m, load_pair(full_halves * (kB / 2) + 2 * ptid, n));
            }
            next_max = m;
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.scan_empty[qb]));
            }
            if (q % kStagesPerTile == kStagesPerTile - 1) {
                if (!reduce_scale(k, next_max)) {
                    return false;
                }
                next_max = 0;
            }
            return true;
        };

        // Producing stage v: finish scan slice v - 1, then convert the raw samples into the FP16
        // planes.
        auto produce = [&](int v) -> bool {
            if (v >= 1 && v - 1 < scan_slices && !consume_slice(v - 1)) {
                return false;
            }
            const int k = v / kStagesPerTile;
            const int st = v % kStagesPerTile;
            const int ex = (k & 1) ? ex_odd : ex_even;
            const float fa = exp2i(ex / 2);
            const float fb = exp2i(ex - ex / 2);
            const int slot = v % S;
            const int rslot = v % kRaw;
            if (!mbar_wait_cluster_bounded(smem_u32(&ctl.empty[slot]), ((v / S) & 1) ^ 1, fault,
                                   kFaultStageEmpty, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.raw_full[rslot]), (v / kRaw) & 1, fault,
                                   kFaultTileLoad, abort)) {
                return false;
            }
            const uint32_t stage = sbase + lay.stages0 + static_cast<uint32_t>(slot) * lay.stage;
            const uint32_t raw = sbase + lay.raw0 + static_cast<uint32_t>(rslot) * lay.raw;
            // Items: (half h, block b, pair q) for 16 float4 (two samples) per window block,
            // enumerated so that a warp covers 4 blocks x 8 pairs of one half: its operand
            // stores then fall in 32 distinct banks.
            const int half_items = lay.rows * 8;
            const long long tail_rel = full_blocks - win0(k);
            const int b_tail =
                tail_rel >= 0 && tail_rel < lay.rows ? static_cast<int>(tail_rel) : -1;
            for (int f = ptid; f < 2 * half_items; f += kProducers) {
                const int h = f >= half_items ? 1 : 0;
                const int g = f - h * half_items;
                const int b = g >> 3;
                const int q = 8 * h + (g & 7);
                float4 v4;
                if (b != b_tail) {
                    v4 = lds128(raw + static_cast<uint32_t>(b * 16 + q) * 16u);  // 0 outside [0, n)
                } else {
                    // The partial last block is outside the tensor maps: plain loads.
                    const long long sidx = full_blocks * kB + 32 * st + 2 * q;
                    v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (sidx + 1 < n) {
                        v4 = __ldg(reinterpret_cast<const float4*>(x + sidx));
                    } else if (sidx < n) {
                        const float2 w2 = __ldg(x + sidx);
                        v4.x = w2.x;
                        v4.y = w2.y;
                    }
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
                mbar_arrive(smem_u32(&ctl.full[slot]));  // forwarded to the even CTA by warp 23
                mbar_arrive(smem_u32(&ctl.raw_empty[rslot]));
            }
            return true;
        };

        bool ok = true;
        if (my_tiles > 0) {
            // Tile 0's scale: this CTA's whole window at once, eight loads in flight per thread.
            const long long lo_s = win0(0) * kB > 0 ? win0(0) * kB : 0;
            const long long end_s = (win0(0) + lay.rows) * kB;
            const long long hi_s = end_s < n ? end_s : n;
            const long long npairs = hi_s > lo_s ? (hi_s - lo_s + 1) / 2 : 0;
            uint32_t m = 0;
            for (long long base = 0; base < npairs; base += 8 * kProducers) {
                uint32_t part[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const long long idx = base + ptid + i * kProducers;
                    part[i] = idx < npairs ? load_pair(lo_s + 2 * idx, hi_s) : 0u;
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    m = max(m, part[i]);
                }
            }
            ok = reduce_scale(0, m);
        }
        for (int v = 0; v < my_steps && ok && !*abort; ++v) {
            ok = produce(v);
        }
    } else if (warp == kTmaWarp) {
        // ---- copy issuer (warp 22, one thread) ----------------------------------------------
        // Scan slice v + sbufs - 2 once slice v - 2 is read, then raw stage v + kRaw once stage
        // v is converted (the first ones were issued during setup).
        if (lane == 0) {
            for (int v = 0; v < my_steps && !*abort; ++v) {
                const int q = v + sbufs - 2;
                if (q < scan_slices) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.scan_empty[q % sbufs]),
                                           ((q / sbufs) & 1) ^ 1, fault, kFaultStageEmpty,
                                           abort)) {
                        break;
                    }
                    issue_scan(q);
                }
                const int vn = v + kRaw;
                if (vn < my_steps) {
                    const int rslot = v % kRaw;
                    if (!mbar_wait_bounded(smem_u32(&ctl.raw_empty[rslot]), (v / kRaw) & 1,
                                           fault, kFaultStageEmpty, abort)) {
                        break;
                    }
                    const uint32_t bar = smem_u32(&ctl.raw_full[rslot]);
                    mbar_arrive_expect_tx(bar, lay.raw);
                    tma_load_2d(sbase + lay.raw0 + static_cast<uint32_t>(rslot) * lay.raw, &xmap,
                                64 * (vn % kStagesPerTile),
                                static_cast<int>(win0(vn / kStagesPerTile)), bar);
                }
            }
        }
    } else if (warp == kMmaWarp && rank == 1 && lane < 3) {
        // ---- forwarders (odd CTA, warp 23, lanes 0-2) ---------------------------------------
        // Each of the odd CTA's hand-off sequences (stage full, H drained, X drained) collects
        // its own warps on the local copy of the barrier; one lane per sequence turns each
        // completed phase into ONE release-arrive on the even CTA's barrier, instead of one
        // cross-CTA arrive per warp. Independent lanes, so no sequence waits behind another.
        if (lane == 0) {
            const uint32_t lead = cluster_map(smem_u32(&ctl.full[0]), 0);
            for (int v = 0; v < my_steps && !*abort; ++v) {
                const int slot = v % S;
                if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (v / S) & 1, fault,
                                       kFaultStageFull, abort)) {
                    break;
                }
                mbar_arrive_cluster(lead + static_cast<uint32_t>(slot) * 8u);
            }
        } else if (lane == 1) {
            const uint32_t lead = cluster_map(smem_u32(&ctl.pempty), 0);
            const int groups = my_tiles * grp.per_tile;
            for (int g = 0; g < groups && !*abort; ++g) {
                if (!mbar_wait_bounded(smem_u32(&ctl.pempty), g & 1, fault, kFaultAccumEmpty,
                                       abort)) {
                    break;
                }
                mbar_arrive_cluster(lead);
            }
        } else {
            const uint32_t lead = cluster_map(smem_u32(&ctl.xempty), 0);
            for (int k = 0; k < my_tiles && !*abort; ++k) {
                if (!mbar_wait_bounded(smem_u32(&ctl.xempty), k & 1, fault, kFaultAccumEmpty,
                                       abort)) {
                    break;
                }
                mbar_arrive_cluster(lead);
            }
        }
    } else if (warp == kMmaWarp && rank == 0 && lane == 0) {
        // ---- MMA issuer for the pair (even CTA, warp 23, one thread) ------------------------
        // Lean issue loop: per MMA one descriptor step and the MMA. The strip descriptor of
        // (K-step st, chunk c) starts 2 st + 32 (C - c) core matrices in, the sample descriptor
        // 2 (C - c) rows into the stage's planes; each next chunk is 256 (strip) and 2 (planes)
        // 16-byte units lower.
        const uint32_t taps_hi = sbase + lay.taps_hi;
        const uint32_t taps_lo = sbase + lay.taps_lo;
        bool stop = false;
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        const uint32_t a_hi0 = (taps_hi >> 4) + static_cast<uint32_t>(32 * C) * 8u;
        const uint32_t a_lo0 = (taps_lo >> 4) + static_cast<uint32_t>(32 * C) * 8u;
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        const uint32_t half_units = (2u * lay.pitch) >> 4;   // second K-step of a stage
        const uint32_t b_base = ((sbase + lay.stages0) >> 4) + static_cast<uint32_t>(2 * C);
        const uint32_t h_acc = tmem;
        const uint32_t x_acc = tmem + kXCol;
        int ready = 0;
        for (int k = 0; k < my_tiles && !stop && !*abort; ++k) {
            for (int gi = 0; gi < grp.per_tile && !stop; ++gi) {
                const int g = k * grp.per_tile + gi;
                int st0, st1, c0, c1;
                h_group_range(grp, P, gi, st0, st1, c0, c1);
                if (!mbar_wait_cluster_bounded(smem_u32(&ctl.pempty), (g & 1) ^ 1, fault,
                                       kFaultAccumEmpty, abort)) {
                    stop = true;
                    break;
                }
                fence_after();
                uint32_t acc = 0;
                for (int st = st0; st < st1; ++st) {
                    const int u = k * kStagesPerTile + st / kStepsPerStage;
                    const int slot = u % S;
                    if (u >= ready) {
                        if (!mbar_wait_cluster_bounded(smem_u32(&ctl.full[slot]), (u / S) & 1, fault,
                                               kFaultStageFull, abort)) {
                            stop = true;
                            break;
                        }
                        fence_after();
                        ready = u + 1;
                    }
                    uint32_t a = a_hi0 + static_cast<uint32_t>(2 * st - 32 * c0) * 8u;
                    uint32_t b = b_base + static_cast<uint32_t>(slot) * stage_units +
                                 static_cast<uint32_t>(st % kStepsPerStage) * half_units -
                                 static_cast<uint32_t>(2 * c0);
                    for (int c = c0; c < c1; ++c) {
                        mma_pair<kIdesc>(h_acc, a_desc | a, b_desc | b, acc);
                        acc = 1;
                        a -= 256;
                        b -= 2;
                    }
                }
                if (stop) {
                    break;
                }
                mma_commit_pair(smem_u32(&ctl.pfull));
                if (gi == 0) {
                    if (!mbar_wait_cluster_bounded(smem_u32(&ctl.xempty), (k & 1) ^ 1, fault,
                                           kFaultAccumEmpty, abort)) {
                        stop = true;
                        break;
                    }
                    fence_after();
                }
                acc = gi == 0 ? 0u : 1u;
                for (int st = st0; st < st1; ++st) {
                    const int slot = (k * kStagesPerTile + st / kStepsPerStage) % S;
                    const uint32_t off = static_cast<uint32_t>(2 * st - 32 * c0) * 8u;
                    uint32_t ah = a_hi0 + off;
                    uint32_t al = a_lo0 + off;
                    uint32_t b = b_base + static_cast<uint32_t>(slot) * stage_units +
                                 static_cast<uint32_t>(st % kStepsPerStage) * half_units -
                                 static_cast<uint32_t>(2 * c0);
                    for (int c = c0; c < c1; ++c) {
                        mma_pair<kIdesc>(x_acc, a_desc | ah, b_desc | (b + split_units), acc);
                        mma_pair<kIdesc>(x_acc, a_desc | al, b_desc | b, 1u);
                        acc = 1;
                        ah -= 256;
                        al -= 256;
                        b -= 2;
                    }
                    if (c1 == P && st % kStepsPerStage == kStepsPerStage - 1) {
                        // Every MMA reading this operand stage has been issued.
                        mma_commit_pair(smem_u32(&ctl.empty[slot]));
                    }
                }
            }
            if (!stop) {
                mma_commit_pair(smem_u32(&ctl.xfull));
            }
        }
        // Every MMA issued has completed before tensor memory is released.
        mma_commit_pair(smem_u32(&ctl.teardown));
        mbar_wait_cluster_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    }

    // After a give-up, TMA copies may still be in flight: give them time to land (bounded).
    if (threadIdx.x == 0 && *abort) {
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
    fence_before();
    __syncthreads();
    cluster_sync_all();   // the pair's MMAs, remote arrivals and copies are all done
    fence_after();
    if (warp == kMmaWarp) {
        tmem_dealloc_pair(tmem, kTmemCols);
    }
}

static bool fits(int num_taps, int stages, int sbufs)
{
    const Layout l = tc2_layout(num_taps, stages, sbufs);
    return l.bytes <= 227u * 1024u && l.rows <= 256 && l.srows <= 256;
}

bool fir_tc2_supported(int num_taps) { return num_taps > 1 && fits(num_taps, 2, 2); }

template <int S>
static cudaError_t launch_pair(const void* x, const float* taps, void* y, long long n,
                               int num_taps, int sbufs, cudaStream_t stream)
{
    const Layout lay = tc2_layout(num_taps, S, sbufs);
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) {
        return err;
    }
    int sms = 0;
    if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
        cudaSuccess) {
        return err;
    }
    // At least 120 KB per CTA keeps one CTA per SM: each pair owns all 512 TMEM columns.
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    cudaFuncAttributes attr{};
    if ((err = cudaFuncGetAttributes(&attr, fir_tc2_kernel<S>)) != cudaSuccess) {
        return err;
    }
    if (attr.maxThreadsPerBlock < kThreads) {
        return cudaErrorLaunchOutOfResources;
    }
    err = cudaFuncSetAttribute(fir_tc2_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    CUtensorMap map;
    CUtensorMap smap;
    err = encode_rows_f32(&map, x, n / kB, 2 * kB, 64, static_cast<uint32_t>(lay.rows));
    if (err == cudaSuccess) {
        err = encode_rows_f32(&smap, x, n / (kB / 2), kB, kB, static_cast<uint32_t>(lay.srows));
    }
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + kB - 1) / kB;
    const int tiles = static_cast<int>((blocks + kNB - 1) / kNB);
    const int npairs = tiles < sms / 2 ? tiles : sms / 2;
    fir_tc2_kernel<S><<<2 * npairs, kThreads, bytes, stream>>>(
        map, smap, static_cast<const float2*>(x), taps, static_cast<float2*>(y), n, num_taps,
        tiles, sbufs);
    return cudaGetLastError();
}

cudaError_t fir_tc2_launch(const void* x, const float* taps, void* y, long long n, int num_taps,
                           int stages, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    if (!fir_tc2_supported(num_taps) || n < kB) {
        return cudaErrorInvalidValue;
    }
    for (int sbufs = kScanBufsMax; sbufs >= 2; sbufs -= 2) {
        if (stages >= 6 && fits(num_taps, 6, sbufs)) {
            return launch_pair<6>(x, taps, y, n, num_taps, sbufs, stream);
        }
        if (stages >= 4 && fits(num_taps, 4, sbufs)) {
            return launch_pair<4>(x, taps, y, n, num_taps, sbufs, stream);
        }
        if (fits(num_taps, 2, sbufs)) {
            return launch_pair<2>(x, taps, y, n, num_taps, sbufs, stream);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t fir_tc2_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_tc2, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_tc2, &zero, sizeof(unsigned int));
}

}  // namespace rfx
