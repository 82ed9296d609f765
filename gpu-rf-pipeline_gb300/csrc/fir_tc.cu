// Tensor-core FIR for sm_103a: the FIR as a block-Toeplitz GEMM on tcgen05, in split FP16.
//
//   y[n] = sum_{k<K} h[k] x[n-k],  x[m < 0] = 0                              (src/fir.cu:1-5)
//
// Blocks of B = 128 outputs: with X[s][j] = x[jB + s] (s < B) the output block j is
//   Y[:, j] = sum_{c=0}^{C} T_c X[:, j - c],   T_c(r, s) = h[cB + r - s]  (0 outside [0, K)),
// C = floor((K + B - 2) / B). One CTA tile is NB = 128 consecutive output blocks (16384 outputs);
// the GEMM per tile is D (128 x 256) += A (128 x 16) B (16 x 256) over K-steps (c, s0):
//
//  * A = T_c restricted to s in [s0, s0 + 16). Output rows are stored reversed (TMEM lane i holds
//    output r = 127 - i); then every 8 x 8 core matrix of A depends only on (row group + K group),
//    so ALL of T_0 .. T_C live in shared memory as one strip of 16C + 31 core matrices,
//    G[t][q][e] = h[(C+1)B - 1 - 8t - q - e], and a K-step's A is a descriptor into that strip
//    with leading- and stride-byte offsets both 128 (the strip is read with overlap).
//  * B = the samples: N index 2j' + {0: I, 1: Q}. Shared memory holds, per K-step pair of
//    8-sample "planes", one 16-byte row per (window block, component); rows are contiguous at a
//    16-byte pitch (stride-byte offset 128 per 8 rows) so the shift by c blocks is just a start
//    address 32c bytes further. Each sample is stored once per tile.
//
// Split precision: x' = 2^ex x and h' = 2^eh h (powers of two chosen per tile and per filter so
// the largest magnitude lands in [2^14, 2^15)), x' = x_hi + x_lo and h' = h_hi + h_lo in FP16,
// and D accumulates h_hi x_hi + h_hi x_lo + h_lo x_hi in FP32 tensor memory; the epilogue scales
// by 2^-(ex+eh) exactly. The dropped h_lo x_lo term and FP32 accumulation keep the normwise
// error near 1e-7 (tests gate it at 2e-6 against the float64 oracle).
//
// Roles (416 threads): warps 0-7 produce (load fp32 samples, find the tile's scale, convert into
// the operand ring), warps 8-11 drain accumulators (TMEM -> registers -> global, one TMEM lane
// quarter each), warp 12 owns tensor memory and issues the MMAs (one thread). Two accumulators
// of 256 columns let the epilogue of one tile overlap the MMAs of the next. Every wait is an
// mbarrier wait bounded in time; a give-up sets the fault word and stops all roles.
#include "fir_tc.cuh"
#include "fir_plain.cuh"
#include "ptx.cuh"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_fir_tc;

namespace {

constexpr int kB = 128;              // outputs per block = MMA M
constexpr int kNB = 128;             // blocks per tile; MMA N = 2 * kNB = 256
constexpr int kN = 2 * kNB;
constexpr int kStagesPerTile = kB / 16;  // K-steps of 16 samples
constexpr int kProducerWarps = 8;
constexpr int kEpilogueWarp0 = 8;
constexpr int kMmaWarp = 12;
constexpr int kThreads = 13 * 32;
constexpr int kProducers = kProducerWarps * 32;
constexpr uint32_t kTmemCols = 512;  // two accumulators of kN columns

constexpr uint32_t kIdesc = (1u << 4)                       // D: F32
                            | (0u << 7) | (0u << 10)        // A, B: F16
                            | (static_cast<uint32_t>(kN >> 3) << 17)
                            | (static_cast<uint32_t>(kB >> 4) << 24);

struct Layout {
    int C;               // previous blocks a block reaches back to
    int W;               // window rows per plane: 2 (kNB + C)
    uint32_t pitch;      // bytes per plane (W * 16 + 16)
    uint32_t split;      // bytes of one split (hi or lo) of a stage: 2 planes
    uint32_t stage;      // bytes per stage: hi + lo
    int tcount;          // core matrices of the tap strip
    uint32_t taps_hi, taps_lo, stages0, bytes;
};

__host__ __device__ inline Layout tc_layout(int num_taps, int stages)
{
    Layout l;
    l.C = (num_taps + kB - 2) / kB;
    l.W = 2 * (kNB + l.C);
    l.pitch = static_cast<uint32_t>(l.W) * 16u + 16u;
    l.split = 2u * l.pitch;
    l.stage = 2u * l.split;
    l.tcount = 16 * l.C + 31;
    l.taps_hi = 1024;
    l.taps_lo = l.taps_hi + 128u * static_cast<uint32_t>(l.tcount);
    l.stages0 = (l.taps_lo + 128u * static_cast<uint32_t>(l.tcount) + 127u) & ~127u;
    l.bytes = l.stages0 + l.stage * static_cast<uint32_t>(stages);
    return l;
}

// Control block at the start of shared memory.
struct Ctrl {
    unsigned long long full[8];
    unsigned long long empty[8];
    unsigned long long tmem_full[2];
    unsigned long long tmem_empty[2];
    unsigned long long scale_full[4];
    unsigned long long reduce[2];
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    int shift[4];             // output exponent shift per tile slot
    uint32_t warp_max[2][kProducerWarps];
    uint32_t tap_max;
};
static_assert(sizeof(Ctrl) <= 1024, "control block");

__device__ __forceinline__ unsigned long long smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<unsigned long long>((addr >> 4) & 0x3FFFu) |
           (static_cast<unsigned long long>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<unsigned long long>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, unsigned long long a,
                                        unsigned long long b, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 2^e as a float for e in [-126, 127].
__device__ __forceinline__ float exp2i(int e)
{
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}

// Exponent that brings a magnitude with these bits into [2^14, 2^15): 141 - biased exponent.
__device__ __forceinline__ int scale_exponent(uint32_t abs_bits)
{
    if (abs_bits == 0) {
        return 0;
    }
    return 141 - static_cast<int>((abs_bits >> 23) & 0xFFu);
}

// hi/lo FP16 split of one value already scaled into range.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void sts32(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

}  // namespace

template <int S>
__global__ void __launch_bounds__(kThreads, 1)
fir_tc_kernel(const float2* __restrict__ x, const float* __restrict__ taps,
              float2* __restrict__ y, long long n, int num_taps, int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const Layout lay = tc_layout(num_taps, S);
    const int C = lay.C;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_fir_tc;

    // ---- setup: barriers, tensor memory, tap strip ----------------------------------------
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kProducerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.tmem_full[i]), 1);
            mbar_init(smem_u32(&ctl.tmem_empty[i]), 4);
            mbar_init(smem_u32(&ctl.reduce[i]), kProducerWarps);
        }
        for (int i = 0; i < 4; ++i) {
            mbar_init(smem_u32(&ctl.scale_full[i]), 1);
        }
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        ctl.tap_max = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&ctl.tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    // Largest tap magnitude (bit pattern of |h|: ordered like the value).
    {
        uint32_t m = 0;
        for (int k = threadIdx.x; k < num_taps; k += kThreads) {
            m = max(m, __float_as_uint(__ldg(taps + k)) & 0x7FFFFFFFu);
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
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (warp < kProducerWarps) {
        // ---- producers ---------------------------------------------------------------------
        const int ptid = threadIdx.x;
        int it = 0;
        for (int tile = blockIdx.x; tile < num_tiles && !*abort; tile += gridDim.x, ++it) {
            const long long j0 = static_cast<long long>(tile) * kNB;
            const long long win0 = (j0 - C) * kB;                       // first window sample
            const long long lo_s = win0 > 0 ? win0 : 0;
            const long long hi_s = (j0 + kNB) * kB < n ? (j0 + kNB) * kB : n;
            // Phase A: the tile's largest |I| or |Q|.
            uint32_t m = 0;
            for (long long s = lo_s + 2 * ptid; s < hi_s; s += 2 * kProducers) {
                if (s + 1 < hi_s) {
                    const float4 v = __ldg(reinterpret_cast<const float4*>(x + s));
                    m = max(m, max(max(__float_as_uint(v.x) & 0x7FFFFFFFu,
                                       __float_as_uint(v.y) & 0x7FFFFFFFu),
                                   max(__float_as_uint(v.z) & 0x7FFFFFFFu,
                                       __float_as_uint(v.w) & 0x7FFFFFFFu)));
                } else {
                    const float2 v = __ldg(x + s);
                    m = max(m, max(__float_as_uint(v.x) & 0x7FFFFFFFu,
                                   __float_as_uint(v.y) & 0x7FFFFFFFu));
                }
            }
            m = __reduce_max_sync(0xFFFFFFFFu, m);
            const int rb = it & 1;
            if (lane == 0) {
                ctl.warp_max[rb][warp] = m;
                mbar_arrive(smem_u32(&ctl.reduce[rb]));
            }
            if (!mbar_wait_bounded(smem_u32(&ctl.reduce[rb]), (it >> 1) & 1, fault,
                                   kFaultStageEmpty, abort)) {
                break;
            }
            uint32_t tmax = 0;
#pragma unroll
            for (int w = 0; w < kProducerWarps; ++w) {
                tmax = max(tmax, ctl.warp_max[rb][w]);
            }
            const int ex = scale_exponent(tmax);
            if (ptid == 0) {
                ctl.shift[it & 3] = -(ex + eh);
                mbar_arrive(smem_u32(&ctl.scale_full[it & 3]));
            }
            const float fa = exp2i(ex / 2);
            const float fb = exp2i(ex - ex / 2);
            // Phase B: one stage per 16-sample K-step.
            const int rows = kNB + C;              // window blocks
            const int items = rows * 8;            // float4 (two samples) per block row
            for (int st = 0; st < kStagesPerTile; ++st) {
                const int g = it * kStagesPerTile + st;
                const int slot = g % S;
                const int s0 = st * 16;
                if (!mbar_wait_bounded(smem_u32(&ctl.empty[slot]), ((g / S) & 1) ^ 1, fault,
                                       kFaultStageEmpty, abort)) {
                    break;
                }
                const uint32_t stage = sbase + lay.stages0 + static_cast<uint32_t>(slot) * lay.stage;
                for (int f = ptid; f < items; f += kProducers) {
                    const int b = f >> 3;
                    const int q = f & 7;
                    const long long sidx = (j0 - C + b) * kB + s0 + 2 * q;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (sidx >= 0 && sidx + 1 < n) {
                        v = __ldg(reinterpret_cast<const float4*>(x + sidx));
                    } else if (sidx >= 0 && sidx < n) {
                        const float2 w = __ldg(x + sidx);
                        v.x = w.x;
                        v.y = w.y;
                    }
                    uint32_t re_hi, re_lo, im_hi, im_lo;
                    split2(v.x * fa * fb, v.z * fa * fb, re_hi, re_lo);
                    split2(v.y * fa * fb, v.w * fa * fb, im_hi, im_lo);
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
            }
        }
    } else if (warp >= kEpilogueWarp0 && warp < kEpilogueWarp0 + 4) {
        // ---- epilogue: TMEM lane quarter (warp % 4) ----------------------------------------
        const int quarter = warp & 3;
        const int lane_row = quarter * 32 + lane;          // TMEM lane = reversed output row
        const int r = kB - 1 - lane_row;                   // output index within the block
        int it = 0;
        for (int tile = blockIdx.x; tile < num_tiles && !*abort; tile += gridDim.x, ++it) {
            const int d = it & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.scale_full[it & 3]), (it >> 2) & 1, fault,
                                   kFaultScale, abort)) {
                break;
            }
            const int shift = ctl.shift[it & 3];
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            if (!mbar_wait_bounded(smem_u32(&ctl.tmem_full[d]), (it >> 1) & 1, fault,
                                   kFaultAccumFull, abort)) {
                break;
            }
            tc_fence_after();
            const long long j0 = static_cast<long long>(tile) * kNB;
            const uint32_t taddr = tmem + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(d * kN);
#pragma unroll 1
            for (int chunk = 0; chunk < kN / 32; ++chunk) {
                uint32_t v[32];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                      "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                      "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
                      "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]),
                      "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr + static_cast<uint32_t>(chunk * 32)));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int b = 0; b < 16; ++b) {
                    const long long o = (j0 + chunk * 16 + b) * kB + r;
                    if (o < n) {
                        y[o] = make_float2(__uint_as_float(v[2 * b]) * fa * fb,
                                           __uint_as_float(v[2 * b + 1]) * fa * fb);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.tmem_empty[d]));
            }
        }
    } else if (warp == kMmaWarp && lane == 0) {
        // ---- MMA issuer ----------------------------------------------------------------------
        const uint32_t taps_hi = sbase + lay.taps_hi;
        const uint32_t taps_lo = sbase + lay.taps_lo;
        int it = 0;
        bool issued = false;
        for (int tile = blockIdx.x; tile < num_tiles && !*abort; tile += gridDim.x, ++it) {
            const int d = it & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.tmem_empty[d]), ((it >> 1) & 1) ^ 1, fault,
                                   kFaultAccumEmpty, abort)) {
                break;
            }
            tc_fence_after();
            const uint32_t dt = tmem + static_cast<uint32_t>(d * kN);
            bool stop = false;
            for (int st = 0; st < kStagesPerTile; ++st) {
                const int g = it * kStagesPerTile + st;
                const int slot = g % S;
                if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (g / S) & 1, fault,
                                       kFaultStageFull, abort)) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t stage = sbase + lay.stages0 + static_cast<uint32_t>(slot) * lay.stage;
                const int s0 = st * 16;
                for (int c = 0; c <= C; ++c) {
                    const uint32_t t0 = static_cast<uint32_t>(16 * (C - c) + s0 / 8) * 128u;
                    const unsigned long long a_hi = smem_desc(taps_hi + t0, 128, 128);
                    const unsigned long long a_lo = smem_desc(taps_lo + t0, 128, 128);
                    const uint32_t row0 = static_cast<uint32_t>(2 * (C - c)) * 16u;
                    const unsigned long long b_hi = smem_desc(stage + row0, lay.pitch, 128);
                    const unsigned long long b_lo = smem_desc(stage + lay.split + row0, lay.pitch, 128);
                    mma_f16(dt, a_hi, b_hi, (st > 0 || c > 0) ? 1u : 0u);
                    mma_f16(dt, a_hi, b_lo, 1u);
                    mma_f16(dt, a_lo, b_hi, 1u);
                    issued = true;
                }
                mma_commit(smem_u32(&ctl.empty[slot]));
            }
            if (stop) {
                break;
            }
            mma_commit(smem_u32(&ctl.tmem_full[d]));
        }
        // Every MMA this thread issued has completed before tensor memory is released.
        mma_commit(smem_u32(&ctl.teardown));
        (void)issued;
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols));
    }
}

bool fir_tc_supported(int num_taps)
{
    return num_taps > 1 && tc_layout(num_taps, 4).bytes <= 227u * 1024u;
}

template <int S>
static cudaError_t launch_stages(const void* x, const float* taps, void* y, long long n,
                                 int num_taps, cudaStream_t stream)
{
    const Layout lay = tc_layout(num_taps, S);
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
    if (lay.bytes > static_cast<uint32_t>(optin)) {
        return cudaErrorInvalidValue;
    }
    // At least 120 KB per block keeps one block per SM: each block owns all 512 TMEM columns.
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    err = cudaFuncSetAttribute(fir_tc_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    const long long blocks = (n + kB - 1) / kB;
    const int tiles = static_cast<int>((blocks + kNB - 1) / kNB);
    const int grid = tiles < sms ? tiles : sms;
    fir_tc_kernel<S><<<grid, kThreads, bytes, stream>>>(
        static_cast<const float2*>(x), taps, static_cast<float2*>(y), n, num_taps, tiles);
    return cudaGetLastError();
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
    if (config.stages >= 6 && tc_layout(num_taps, 6).bytes <= 227u * 1024u) {
        return launch_stages<6>(x, taps, y, n, num_taps, stream);
    }
    return launch_stages<4>(x, taps, y, n, num_taps, stream);
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
    for (int c = 0; c < count; ++c) {
        if (captures[c].num_samples == 0) {
            continue;
        }
        const bool tc = impl == RFX_FIR_TC && fir_tc_supported(captures[c].num_taps);
        cudaError_t err = tc ? fir_tc_launch(captures[c].x, captures[c].taps, captures[c].y,
                                             captures[c].num_samples, captures[c].num_taps,
                                             TcConfig{kNB, 4}, stream)
                             : fir_plain_launch(captures[c].x, captures[c].taps, captures[c].y,
                                                captures[c].num_samples, captures[c].num_taps,
                                                stream);
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
}

}  // namespace rfx
