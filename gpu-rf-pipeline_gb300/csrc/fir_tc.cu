// Tensor-core FIR for sm_103a: the FIR as a block-Toeplitz GEMM on tcgen05, in split FP16.
//
//   y[n] = sum_{k<K} h[k] x[n-k],  x[m < 0] = 0                              (src/fir.cu:1-5)
//
// Blocks of B = 128 outputs: with X[s][j] = x[jB + s] (s < B) the output block j is
//   Y[:, j] = sum_{c=0}^{C} T_c X[:, j - c],   T_c(r, s) = h[cB + r - s]  (0 outside [0, K)),
// C = floor((K + B - 2) / B). One tile is NB = 96 consecutive output blocks (12288 outputs);
// per tile the GEMM is D (128 x 192) += A (128 x 16) B (16 x 192) over K-steps (c, s0):
//
//  * A = T_c restricted to s in [s0, s0 + 16). Output rows are stored reversed (TMEM lane i holds
//    output r = 127 - i); then every 8 x 8 core matrix of A depends only on (row group + K group),
//    so ALL of T_0 .. T_C live in shared memory as one strip of 16C + 31 core matrices,
//    G[t][q][e] = h[(C+1)B - 1 - 8t - q - e], and a K-step's A is a descriptor into that strip
//    with leading- and stride-byte offsets both 128 (the strip is read with overlap).
//  * B = the samples: N index 2j' + {0: I, 1: Q}. Shared memory holds, per K-step, two 8-sample
//    "planes" with one 16-byte row per (window block, component); rows are contiguous at a
//    16-byte pitch (stride-byte offset 128 per 8 rows), so the shift by c blocks is a start
//    address 32c bytes further. Each sample is converted once per tile.
//
// Split precision: x' = 2^ex x and h' = 2^eh h (powers of two chosen per tile and per filter so
// the largest magnitude lands in [2^14, 2^15)), x' = x_hi + x_lo and h' = h_hi + h_lo in FP16,
// and the MMAs sum h_hi x_hi + h_hi x_lo + h_lo x_hi with FP32 accumulation; the result is
// scaled by 2^-(ex+eh) exactly.
//
// Accumulation: the tensor core adds each MMA's products into its FP32 accumulator with
// round-toward-zero, so the error of an accumulator grows with the number of MMAs it takes, in
// units of its own magnitude. The large product h_hi x_hi therefore goes to accumulator H in
// GROUPS of at most 18 MMAs (whole K-steps; at 1025 taps two K-steps of 9 chunks); the worker
// warps add each group's sum into FP32 running sums in registers (round-to-nearest). The two
// cross products, 2^-11 smaller, go to accumulator X for the whole tile and are drained once.
// Per group the MMA thread issues the H MMAs, commits, then the group's X MMAs (twice as many),
// during which the workers drain H. Larger groups mean fewer commits and hand-offs for the
// issuing thread (which bounds the MMA rate) at an error that grows with the group: 5e-7 at 9
// MMAs, 8e-7 at 18 (1025 taps).
//
// Roles (768 threads): warps 0-15 hold the running sums: a drain warp w drains TMEM lane quarter
// w % 4, columns 48 (w / 4) .. +47 of H and of X, and writes those outputs (48 running sums per
// thread); warps 16-22 produce: each K-step's fp32 samples arrive by a 2-D TMA copy (zero fill
// outside the input) and are converted into the FP16 planes, the next tile's scale is a max
// over its input window, copied by TMA in eight slices three K-steps ahead; warp 23 owns tensor
// memory and issues the MMAs (one thread). The drains never wait behind production, and the
// producer count balances the MMA rate (measured: 3 producer warps 173 us, 5 154 us, 7 144 us at
// 1025 taps; beyond 7 no gain). 24 warps: one SM sub-partition holds six, so 80 registers.
// Every wait is an mbarrier wait bounded in time; a give-up sets the fault word and every role
// stops.
#include "fir_tc.cuh"
#include "fir_plain.cuh"
#include "fir_tc2.cuh"
#include "tuning.hpp"
#include "sample_fmt.cuh"
#include "tc_common.cuh"
#include "tmap.hpp"

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

namespace rfx {

static __device__ unsigned int g_fault_fir_tc;

namespace {

using namespace tc;

constexpr int kB = 128;                  // outputs per block = MMA M
constexpr int kNB = 96;                  // blocks per tile; MMA N = 2 * kNB = 192
constexpr int kN = 2 * kNB;
constexpr int kStagesPerTile = kB / 16;  // K-steps of 16 samples
constexpr int kDrainWarps = 16;          // hold the running sums, drain, store
constexpr int kProducerWarps = 7;        // scan, convert, issue the copies
constexpr int kProducers = kProducerWarps * 32;
constexpr int kFirstProducerWarp = kDrainWarps;
constexpr int kMmaWarp = kDrainWarps + kProducerWarps;
constexpr int kThreads = (kMmaWarp + 1) * 32;
constexpr int kCols = kN / 4;            // running sums per worker thread
constexpr int kHGroup = 18;              // MMAs per H accumulation, at most
constexpr int kRaw = 3;                  // TMA raw-sample ring depth
constexpr int kScanBufsMax = 4;          // scan slice ring depth: 4 (2 for the longest filters);
                                         // slices are copied depth - 1 K-steps ahead
constexpr uint32_t kTmemCols = 512;      // H (kN columns) and X (kN columns), 384 used
constexpr uint32_t kXCol = kN;           // first column of X
constexpr uint32_t kIdesc = idesc_f16(kB, kN);

struct Layout {
    int C;               // previous blocks a block reaches back to
    int rows;            // window blocks per tile: kNB + C
    int srows;           // window rows per scan slice: ceil(rows / 8)
    uint32_t pitch;      // bytes per plane (2 rows * 16 B per block + 16)
    uint32_t split;      // bytes of one split (hi or lo) of a stage: 2 planes
    uint32_t stage;      // bytes per operand stage: hi + lo
    uint32_t raw_tx;     // bytes one raw copy delivers: rows * 32 components * es
    uint32_t scan_tx;    // bytes one scan copy delivers: srows * 256 components * es
    uint32_t raw;        // raw stage pitch (raw_tx rounded up to 128 B)
    uint32_t scan;       // scan slice pitch (scan_tx rounded up to 128 B)
    int tcount;          // core matrices of the tap strip
    int sbufs;           // scan slice buffers
    uint32_t taps_hi, taps_lo, raw0, scan0, stages0, bytes;
};

// es: bytes per input component (4 cf32, 2 ci16, 1 ci8).
__host__ __device__ inline Layout tc_layout(int num_taps, int stages, int sbufs, int es = 4)
{
    Layout l;
    l.sbufs = sbufs;
    l.C = (num_taps + kB - 2) / kB;
    l.rows = kNB + l.C;
    l.srows = (l.rows + kStagesPerTile - 1) / kStagesPerTile;
    l.pitch = static_cast<uint32_t>(2 * l.rows) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    // Each copy's destination 128-byte aligned.
    l.raw_tx = static_cast<uint32_t>(l.rows) * 32u * static_cast<uint32_t>(es);
    l.scan_tx = static_cast<uint32_t>(l.srows) * 256u * static_cast<uint32_t>(es);
    l.raw = (l.raw_tx + 127u) & ~127u;
    l.scan = (l.scan_tx + 127u) & ~127u;
    l.tcount = 16 * l.C + 31;
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount);
    l.raw0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount) + 127u) & ~127u;
    l.scan0 = l.raw0 + kRaw * l.raw;
    l.stages0 = l.scan0 + static_cast<uint32_t>(sbufs) * l.scan;
    l.bytes = l.stages0 + l.stage * static_cast<uint32_t>(stages);
    return l;
}

// Control block at the start of shared memory.
struct Ctrl {
    unsigned long long full[8];
    unsigned long long empty[8];
    unsigned long long raw_full[kRaw];
    unsigned long long raw_empty[kRaw];
    unsigned long long scan_full[kScanBufsMax];
    unsigned long long scan_empty[kScanBufsMax];
    unsigned long long pfull;     // H group summed (tcgen05.commit)
    unsigned long long pempty;    // H drained (every drain warp)
    unsigned long long xfull;     // X of a tile summed
    unsigned long long xempty;    // X drained
    unsigned long long sready[4]; // the scale of tile k is in ex[k % 4]
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t pmax[2][kProducerWarps];
    int ex[4];
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

// H groups of a tile. For P <= 18 chunks a group is `ksg` whole K-steps (at most 18 MMAs, and
// fewer K-steps than operand stages, since a group holds its stages until its X MMAs); for
// P > 18 each K-step splits into `gpk` groups of at most `cpg` chunks.
struct HGroups {
    int ksg;        // K-steps per group (P <= 18)
    int gpk;        // groups per K-step (P > 18), else 1
    int cpg;        // chunks per group (P > 18), else P
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

// K-steps [st0, st1) and chunks [c0, c1) of group gi of a tile.
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

// xmap: x as rows of 256 components (one block), boxes of 32 components x `rows` (one K-step's
// samples of a tile window). smap: the same rows, boxes of 256 components x `srows` (a scan
// slice). fmt: x's sample format (0 cf32, 1 ci16, 2 ci8); the copies move the components as
// stored and the producers decode them.
// kInt: x holds integer components (fmt 1 or 2, a runtime argument); without it x is cf32
// and the format branches compile away (they cost the cf32 kernel 7 %).
template <int S, bool kInt>
__global__ void __launch_bounds__(kThreads, 1)
fir_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap smap,
              const void* __restrict__ x, const float* __restrict__ taps,
              float2* __restrict__ y, long long n, int num_taps, int num_tiles, int sbufs, int fmt)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    if (!kInt) {
        fmt = 0;
    }
    const int es = component_bytes(fmt);
    const Layout lay = tc_layout(num_taps, S, sbufs, es);
    const int C = lay.C;
    const int P = C + 1;                       // chunks per K-step
    const HGroups grp = h_groups(P, S);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_tc;
    // This block's tiles: blockIdx.x, + gridDim.x, ...; its K-steps are numbered u = 8 k + st.
    const int my_tiles = static_cast<int>(blockIdx.x) < num_tiles
                             ? (num_tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                             : 0;
    const int my_steps = my_tiles * kStagesPerTile;
    const int scan_slices = my_tiles > 1 ? (my_tiles - 1) * kStagesPerTile : 0;
    const long long full_blocks = n / kB;      // rows the tensor maps cover
    auto tile_of = [&](int k) { return static_cast<int>(blockIdx.x) + k * gridDim.x; };

    // ---- setup: barriers, tensor memory, first raw copies, tap strip -----------------------
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < kRaw; ++i) {
            mbar_init(smem_u32(&ctl.raw_full[i]), 1);
            mbar_init(smem_u32(&ctl.raw_empty[i]), kProducerWarps);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(smem_u32(&ctl.sready[i]), 1);
        }
        for (int i = 0; i < sbufs; ++i) {
            mbar_init(smem_u32(&ctl.scan_full[i]), 1);
            mbar_init(smem_u32(&ctl.scan_empty[i]), kProducerWarps);
        }
        mbar_init(smem_u32(&ctl.pfull), 1);
        mbar_init(smem_u32(&ctl.pempty), kDrainWarps);
        mbar_init(smem_u32(&ctl.xfull), 1);
        mbar_init(smem_u32(&ctl.xempty), kDrainWarps);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        ctl.tap_max = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    __syncthreads();
    // Scan slice q: the next tile's (q / 8 + 1) window rows (q % 8) srows .. + srows.
    auto issue_scan = [&](int q) {
        const int kn = q / kStagesPerTile + 1;
        const uint32_t bar = smem_u32(&ctl.scan_full[q % sbufs]);
        mbar_arrive_expect_tx(bar, lay.scan_tx);
        tma_load_2d(sbase + lay.scan0 + static_cast<uint32_t>(q % sbufs) * lay.scan, &smap,
                    0, tile_of(kn) * kNB - C + (q % kStagesPerTile) * lay.srows, bar);
    };
    // Raw sample stages 0 .. kRaw-1 (K-step u: rows from block 128 k - C, floats 32 (u % 8)..)
    // and the first scan slices.
    if (threadIdx.x == 0) {
        for (int u = 0; u < kRaw && u < my_steps; ++u) {
            const uint32_t bar = smem_u32(&ctl.raw_full[u]);
            mbar_arrive_expect_tx(bar, lay.raw_tx);
            tma_load_2d(sbase + lay.raw0 + u * lay.raw, &xmap, 32 * (u % kStagesPerTile),
                        tile_of(u / kStagesPerTile) * kNB - C, bar);
        }
        for (int q = 0; q < sbufs - 2 && q < scan_slices; ++q) {
            issue_scan(q);
        }
    }
    // Largest tap magnitude (bit pattern of |h|: ordered like the value).
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
        const int dmax = (C + 1) * kB - 1;
        // Two adjacent elements e, e+1 of core matrix t, row q per iteration.
        const int pairs = lay.tcount * 32;
        for (int i = threadIdx.x; i < pairs; i += kThreads) {
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

    if (warp < kDrainWarps) {
        // ---- drain warps: running sums, outputs ----------------------------------------------
        const int quarter = warp & 3;
        const int slice = warp >> 2;                       // columns kCols * slice .. +kCols-1
        const int r = kB - 1 - (quarter * 32 + lane);      // output row of this TMEM lane
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(slice * kCols);
        float acc[kCols];
#pragma unroll
        for (int i = 0; i < kCols; ++i) {
            acc[i] = 0.0f;
        }
        // Adds accumulator columns col .. col + kCols - 1 of this lane into acc.
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
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            for (int gi = 0; gi < grp.per_tile; ++gi, ++g) {
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
            // The tile's sample scale (written by the producers before its first K-step).
            if (!mbar_wait_bounded(smem_u32(&ctl.sready[k & 3]), (k >> 2) & 1, fault,
                                   kFaultScale, abort)) {
                break;
            }
            const int ex = *reinterpret_cast<volatile int*>(&ctl.ex[k & 3]);
            const int shift = -(ex + eh);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
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
        // ---- producers: scales, operand stages, copies ---------------------------------------
        const int pw = warp - kFirstProducerWarp;
        const int ptid = static_cast<int>(threadIdx.x) - kFirstProducerWarp * 32;
        int ex_even = 0;                                   // scale exponents of even, odd tiles
        int ex_odd = 0;
        uint32_t next_max = 0;                             // running max of the next tile's scan

        // Max of |samples| in [s, s + 2) clipped to hi_s (plain loads, for the partial block).
        auto load_pair = [&](long long s, long long hi_s) -> uint32_t {
            if (s + 1 < hi_s) {
                return absmax4(ldg_pair(x, fmt, s));
            }
            if (s < hi_s) {
                const float2 w2 = ldg_one(x, fmt, s);
                return max(absbits(w2.x), absbits(w2.y));
            }
            return 0u;
        };
        // Combines the producers' partial maxima for tile k into its scale exponent and
        // publishes it to the drain warps.
        auto reduce_scale = [&](int k, uint32_t m) {
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
            // Clamped to 127 (only a window with max |x| < 2^-113 would want more), so that 2^ex
            // is one float and the producers scale with a single exact multiply.
            const int ex = min(scale_exponent(tmax), 127);
            if (k & 1) {
                ex_odd = ex;
            } else {
                ex_even = ex;
            }
            if (ptid == 0) {
                ctl.ex[k & 3] = ex;
                mbar_arrive(smem_u32(&ctl.sready[k & 3]));
            }
        };
        // Scan slice q, copied by TMA sbufs - 1 K-steps earlier: rows past the window are
        // ignored; the partial last block lies outside the tensor map (the copy reads zeros
        // there) and is read from global memory.
        auto consume_slice = [&](int q) -> bool {
            const int qb = q % sbufs;
            if (!mbar_wait_bounded(smem_u32(&ctl.scan_full[qb]), (q / sbufs) & 1, fault,
                                   kFaultTileLoad, abort)) {
                return false;
            }
            const int k = q / kStagesPerTile + 1;
            const long long j0 = static_cast<long long>(tile_of(k)) * kNB;
            const int r0 = (q % kStagesPerTile) * lay.srows;
            const uint32_t buf = sbase + lay.scan0 + static_cast<uint32_t>(qb) * lay.scan;
            const int quads = min(lay.srows, lay.rows - r0) * 64;   // sample pairs in the window
            const uint32_t pair_bytes = 4u * static_cast<uint32_t>(es);
            uint32_t m = next_max;
#pragma unroll 4
            for (int f = ptid; f < quads; f += kProducers) {
                m = max(m, absmax4(lds_pair(buf + static_cast<uint32_t>(f) * pair_bytes, fmt)));
            }
            const long long tail_row = full_blocks - (j0 - C) - r0;
            if (tail_row >= 0 && tail_row * 64 < quads && ptid < 64) {
                m = max(m, load_pair(full_blocks * kB + 2 * ptid, n));
            }
            next_max = m;
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.scan_empty[qb]));
            }
            if (q % kStagesPerTile == kStagesPerTile - 1) {
                reduce_scale(k, next_max);
                next_max = 0;
            }
            return true;
        };

        // Producing K-step v: finish scan slice v - 1, convert the raw samples into the FP16
        // planes, then queue step v + kRaw's raw copy and scan slice v + sbufs - 2.
        auto produce = [&](int v) -> bool {
            if (v >= 1 && v - 1 < scan_slices && !consume_slice(v - 1)) {
                return false;
            }
            const int k = v / kStagesPerTile;
            const int st = v % kStagesPerTile;
            const long long j0 = static_cast<long long>(tile_of(k)) * kNB;
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
            const uint32_t pair_bytes = 4u * static_cast<uint32_t>(es);
            // Window row of the input's last, partial block (outside the tensor maps), if any.
            const long long tail_rel = full_blocks - (j0 - C);
            const int b_tail = tail_rel >= 0 && tail_rel < lay.rows ? static_cast<int>(tail_rel) : -1;
            // Item f = 8 b + q (sample pair q of window row b): kProducers is a multiple of 8, so
            // a thread keeps its q and steps b by kProducers / 8.
            static_assert(kProducers % 8 == 0, "producer stride");
            const int q = ptid & 7;
            const uint32_t elem_off = static_cast<uint32_t>(q >> 2) * lay.pitch +
                                      static_cast<uint32_t>(q & 3) * 4u;
#pragma unroll 2
            for (int b = ptid >> 3; b < lay.rows; b += kProducers / 8) {
                const int f = 8 * b + q;
                float4 v4;
                if (b != b_tail) {
                    // zero outside [0, n)
                    v4 = lds_pair(raw + static_cast<uint32_t>(f) * pair_bytes, fmt);
                } else {
                    // The partial block: plain loads.
                    const long long sidx = full_blocks * kB + 16 * st + 2 * q;
                    v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (sidx + 1 < n) {
                        v4 = ldg_pair(x, fmt, sidx);
                    } else if (sidx < n) {
                        const float2 w2 = ldg_one(x, fmt, sidx);
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
                // Refill this raw slot with K-step v + kRaw once every producer has converted it.
                if (v + kRaw < my_steps) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.raw_empty[rslot]), (v / kRaw) & 1,
                                           fault, kFaultStageEmpty, abort)) {
                        return false;
                    }
                    const int vn = v + kRaw;
                    const uint32_t bar = smem_u32(&ctl.raw_full[rslot]);
                    mbar_arrive_expect_tx(bar, lay.raw_tx);
                    tma_load_2d(raw, &xmap, 32 * (vn % kStagesPerTile),
                                tile_of(vn / kStagesPerTile) * kNB - C, bar);
                }
                // Scan slice q into its buffer once slice q - sbufs is read.
                const int q = v + sbufs - 2;
                if (q < scan_slices) {
                    if (!mbar_wait_bounded(smem_u32(&ctl.scan_empty[q % sbufs]),
                                           ((q / sbufs) & 1) ^ 1, fault, kFaultStageEmpty,
                                           abort)) {
                        return false;
                    }
                    issue_scan(q);
                }
            }
            return true;
        };

        bool ok = true;
        if (my_tiles > 0) {
            // Tile 0's scale: its whole window at once, eight loads in flight per thread.
            const long long j0 = static_cast<long long>(tile_of(0)) * kNB;
            const long long win0 = (j0 - C) * kB;
            const long long lo0 = win0 > 0 ? win0 : 0;
            const long long hi0 = (j0 + kNB) * kB < n ? (j0 + kNB) * kB : n;
            const long long pairs = (hi0 - lo0 + 1) / 2;
            uint32_t m = 0;
            for (long long base = 0; base < pairs; base += 8 * kProducers) {
                uint32_t part[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const long long idx = base + ptid + i * kProducers;
                    part[i] = idx < pairs ? load_pair(lo0 + 2 * idx, hi0) : 0u;
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    m = max(m, part[i]);
                }
            }
            reduce_scale(0, m);
        }
        for (int v = 0; v < my_steps && ok && !*abort; ++v) {
            ok = produce(v);
        }
    } else if (warp == kMmaWarp && lane == 0) {
        // ---- MMA issuer (warp 23, one thread) ----------------------------------------------
        const uint32_t taps_hi = sbase + lay.taps_hi;
        const uint32_t taps_lo = sbase + lay.taps_lo;
        // The issue loop is latency-bound in this one thread, so it is kept lean: per MMA one
        // descriptor step and the MMA. Descriptors differ only in their start-address field
        // (address / 16): the tap strip descriptor of (K-step st, chunk c) starts
        // 16 (C - c) + 2 st core matrices in, the sample descriptor 2 (C - c) rows into the
        // stage's planes; each next chunk is 128 (strip) and 2 (planes) units lower.
        bool stop = false;
        const unsigned long long a_desc = smem_desc(0, 128, 128);
        const unsigned long long b_desc = smem_desc(0, lay.pitch, 128);
        const uint32_t a_hi0 = (taps_hi >> 4) + static_cast<uint32_t>(16 * C) * 8u;
        const uint32_t a_lo0 = (taps_lo >> 4) + static_cast<uint32_t>(16 * C) * 8u;
        const uint32_t stage_units = lay.stage >> 4;
        const uint32_t split_units = lay.split >> 4;
        const uint32_t b_base = ((sbase + lay.stages0) >> 4) + static_cast<uint32_t>(2 * C);
        const uint32_t h_acc = tmem;
        const uint32_t x_acc = tmem + kXCol;
        int ready = 0;        // K-steps (block-wide numbering) whose stage has been waited for
        for (int k = 0; k < my_tiles && !stop && !*abort; ++k) {
            for (int gi = 0; gi < grp.per_tile && !stop; ++gi) {
                const int g = k * grp.per_tile + gi;
                int st0, st1, c0, c1;
                h_group_range(grp, P, gi, st0, st1, c0, c1);
                // H is free once the workers drained the previous group.
                if (!mbar_wait_bounded(smem_u32(&ctl.pempty), (g & 1) ^ 1, fault,
                                       kFaultAccumEmpty, abort)) {
                    stop = true;
                    break;
                }
                fence_after();
                // Pass 0: h_hi x_hi into H.
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
                    // 64-bit descriptors stepped in their start-address field (no borrow
                    // leaves it: addresses stay positive).
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
                // Pass 1: h_hi x_lo + h_lo x_hi into X, zeroed at the tile's first MMA.
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
                        // Every MMA reading this K-step's operand stage has been issued.
                        mma_commit(smem_u32(&ctl.empty[slot]));
                    }
                }
            }
            if (!stop) {
                mma_commit(smem_u32(&ctl.xfull));
            }
        }
        // Every MMA this thread issued has completed before tensor memory is released.
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
    if (warp == kMmaWarp) {
        tmem_dealloc(tmem, kTmemCols);
    }
}

bool fir_tc_supported(int num_taps)
{
    const Layout l = tc_layout(num_taps, 2, 2);
    return num_taps > 1 && l.bytes <= 227u * 1024u && l.rows <= 256;
}

template <int S, bool kInt>
static cudaError_t launch_stages(int fmt, const void* x, const float* taps, void* y, long long n,
                                 int num_taps, int sbufs, cudaStream_t stream)
{
    const int es = component_bytes(fmt);
    const Layout lay = tc_layout(num_taps, S, sbufs, es);
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
    // The block's warps must fit the register file at this register count.
    cudaFuncAttributes attr{};
    if ((err = cudaFuncGetAttributes(&attr, fir_tc_kernel<S, kInt>)) != cudaSuccess) {
        return err;
    }
    if (attr.maxThreadsPerBlock < kThreads) {
        return cudaErrorLaunchOutOfResources;
    }
    err = cudaFuncSetAttribute(fir_tc_kernel<S, kInt>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    // x viewed as rows of 256 components (one 128-sample block per row), full blocks only;
    // boxes of 32 components (16 samples) by the tile's window rows.
    CUtensorMap map;
    CUtensorMap smap;
    err = encode_rows(&map, x, es, n / kB, 2 * kB, 32, static_cast<uint32_t>(lay.rows));
    if (err == cudaSuccess) {
        err = encode_rows(&smap, x, es, n / kB, 2 * kB, 2 * kB, static_cast<uint32_t>(lay.srows));
    }
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + kB - 1) / kB;
    const int tiles = static_cast<int>((blocks + kNB - 1) / kNB);
    const int grid = tiles < sms ? tiles : sms;
    fir_tc_kernel<S, kInt><<<grid, kThreads, bytes, stream>>>(
        map, smap, x, taps, static_cast<float2*>(y), n, num_taps, tiles, sbufs, fmt);
    return cudaGetLastError();
}

// The single-CTA form over x in format fmt (n >= one block).
static cudaError_t launch_single(int fmt, const void* x, const float* taps, void* y, long long n,
                                 int num_taps, int max_stages, cudaStream_t stream)
{
    const int es = component_bytes(fmt);
    // The deep scan ring first (it hides the scan copies' latency), then the most stages.
    for (int sbufs = kScanBufsMax; sbufs >= 2; sbufs -= 2) {
        if (max_stages >= 6 && tc_layout(num_taps, 6, sbufs, es).bytes <= 227u * 1024u) {
            return fmt == 0 ? launch_stages<6, false>(fmt, x, taps, y, n, num_taps, sbufs, stream)
                            : launch_stages<6, true>(fmt, x, taps, y, n, num_taps, sbufs, stream);
        }
        if (max_stages >= 4 && tc_layout(num_taps, 4, sbufs, es).bytes <= 227u * 1024u) {
            return fmt == 0 ? launch_stages<4, false>(fmt, x, taps, y, n, num_taps, sbufs, stream)
                            : launch_stages<4, true>(fmt, x, taps, y, n, num_taps, sbufs, stream);
        }
        if (tc_layout(num_taps, 2, sbufs, es).bytes <= 227u * 1024u) {
            return fmt == 0 ? launch_stages<2, false>(fmt, x, taps, y, n, num_taps, sbufs, stream)
                            : launch_stages<2, true>(fmt, x, taps, y, n, num_taps, sbufs, stream);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t fir_tc_launch(const void* x, const float* taps, void* y, long long n, int num_taps,
                          TcConfig config, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    if (!fir_tc_supported(num_taps)) {
        return cudaErrorInvalidValue;
    }
    if (config.tile_blocks == kTcPairTile && n >= 2 * kB && fir_tc2_supported(num_taps)) {
        return fir_tc2_launch(x, taps, y, n, num_taps, config.stages, stream);
    }
    if (n < kB) {
        // Shorter than one block: the tensor map would be empty; the plain kernel is exact.
        return fir_plain_launch(x, taps, y, n, num_taps, stream);
    }
    if (config.tile_blocks == kTcWindowTile && fir_tcw_supported(num_taps)) {
        return fir_tcw_launch(0, x, taps, y, n, num_taps, stream);
    }
    return launch_single(0, x, taps, y, n, num_taps, config.stages, stream);
}

cudaError_t fir_tc_launch_format(int format, const void* x, const float* taps, void* y,
                                 long long n, int num_taps, TcConfig config, cudaStream_t stream)
{
    if (format == 0) {
        return fir_tc_launch(x, taps, y, n, num_taps, config, stream);
    }
    if (format != 1 && format != 2) {
        return cudaErrorInvalidValue;
    }
    if (n <= 0) {
        return cudaSuccess;
    }
    if (!fir_tc_supported(num_taps)) {
        return cudaErrorInvalidValue;
    }
    if (n < kB) {
        return fir_plain_launch_format(format, x, taps, y, n, num_taps, stream);
    }
    if (config.tile_blocks == kTcWindowTile && fir_tcw_supported(num_taps)) {
        return fir_tcw_launch(format, x, taps, y, n, num_taps, stream);
    }
    // Otherwise integer input runs in the single-CTA form (also where cf32 runs the pair form).
    return launch_single(format, x, taps, y, n, num_taps,
                         config.tile_blocks == kTcPairTile ? 6 : config.stages, stream);
}

long long fir_tc_tile_outputs(int num_taps, long long n, TcConfig config)
{
    if (n <= 0 || !fir_tc_supported(num_taps)) {
        return 1;
    }
    if (config.tile_blocks == kTcPairTile && n >= 2 * kB && fir_tc2_supported(num_taps)) {
        return 96LL * 256;
    }
    if (n >= kB && config.tile_blocks == kTcWindowTile && fir_tcw_supported(num_taps)) {
        return fir_tcw_tile_outputs();
    }
    return n < kB ? 1 : static_cast<long long>(kNB) * kB;
}

long long fir_tc_tile_outputs_format(int format, int num_taps, long long n, TcConfig config)
{
    if (format == 0) {
        return fir_tc_tile_outputs(num_taps, n, config);
    }
    if (n <= 0 || n < kB || !fir_tc_supported(num_taps)) {
        return 1;
    }
    return config.tile_blocks == kTcWindowTile && fir_tcw_supported(num_taps)
               ? fir_tcw_tile_outputs()
               : static_cast<long long>(kNB) * kB;
}

cudaError_t fir_tc_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_tc, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_tc, &zero, sizeof(unsigned int));
}

cudaError_t fir_batch_launch(int impl, const rfx_fir_capture* captures, int count,
                             cudaStream_t stream)
{
    if (impl == RFX_FIR_TC) {
        return fir_batch_tc_launch(captures, count, stream);
    }
    if (impl == RFX_FIR_AUTO) {
        // Each capture where the tuned rule puts it: the tensor-core captures in one persistent
        // launch, the others in one plain launch per 256 captures.
        std::vector<rfx_fir_capture> tc;
        PlainCaps* plain = new PlainCaps{};
        cudaError_t err = cudaSuccess;
        auto flush = [&]() {
            if (plain->count > 0 && err == cudaSuccess) {
                err = fir_plain_caps_launch(*plain, stream);
            }
            plain->count = 0;
            plain->tile0[0] = 0;
        };
        for (int c = 0; c < count && err == cudaSuccess; ++c) {
            const rfx_fir_capture& cap = captures[c];
            if (cap.num_samples == 0) {
                continue;
            }
            if (tuned_fir_batch_launch_impl(cap.num_taps, cap.num_samples) == RFX_FIR_TC) {
                tc.push_back(cap);
                continue;
            }
            const int i = plain->count;
            plain->x[i] = cap.x;
            plain->y[i] = cap.y;
            plain->taps[i] = cap.taps;
            plain->num_samples[i] = cap.num_samples;
            plain->num_taps[i] = cap.num_taps;
            plain->tile0[i + 1] = plain->tile0[i] + static_cast<int>((cap.num_samples +
                                                                       kPlainTileOutputs - 1) /
                                                                      kPlainTileOutputs);
            plain->count = i + 1;
            if (plain->count == kPlainCapsMax) {
                flush();
            }
        }
        flush();
        delete plain;
        if (err != cudaSuccess) {
            return err;
        }
        return tc.empty() ? cudaSuccess
                          : fir_batch_tc_launch(tc.data(), static_cast<int>(tc.size()), stream);
    }
    // The plain kernel: one launch per capture, as the project runs a batch.
    for (int c = 0; c < count; ++c) {
        if (captures[c].num_samples == 0) {
            continue;
        }
        const cudaError_t err = fir_plain_launch(captures[c].x, captures[c].taps, captures[c].y,
                                                 captures[c].num_samples, captures[c].num_taps,
                                                 stream);
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
}

}  // namespace rfx
