// Tensor-core polyphase channelizer for sm_103a, M = 64 channels, one fused kernel.
//
//   u[t][m] = sum_p h[pM + m] x[tM - pM - m]            (x[i < 0] = 0)      src/channelize.cu:25-49
//   z[t][k] = sum_m u[t][m] e^{+2 pi i k m / M}                              src/channelize.cu:70-71
//
// Per tile of 128 frames (8192 samples):
//  1. Branch sums on CUDA cores, FP32: a thread owns branches 2j, 2j+1 for 8 consecutive
//     frames. For one branch the frames form a FIR over the decimated sequence
//     s_d = x[(t0 + d) M - m] with taps g_p = h[pM + m]; eight outputs per thread come from two
//     alternating 8-sample register blocks (no moves), taps in ascending p, one packed f32x2
//     fused multiply-add per tap — the arithmetic order of the project's branch kernel.
//  2. The tile's largest |u| sets a power-of-two scale; u' = u_hi + u_lo in FP16 is written as
//     the GEMM's A operand (rows = frames, K = [Re u[0..63], Im u[0..63]]).
//  3. The DFT as a real GEMM: [Re z, Im z] (128 x 128) = A (128 x 128) W, with
//     W = [[cos, sin], [-sin, cos]](2 pi k m / M) built in FP64 on the GPU (rfx_chan_plan_create)
//     and split hi/lo once; three split products per K-step on tcgen05 (M=128, N=128, K=16).
//     The round-toward-zero FP32 accumulation is kept short: four TMEM accumulators take six
//     MMAs each and are summed in FP32 registers.
//  4. Scale back by 2^-(eu + ew) and store each frame's 64 channels.
//
// Roles (544 threads): warps 0-15 compute branch sums, write operands, and drain the
// accumulators (warp w: TMEM lane quarter w % 4 = frames 32 (w % 4) .. +31, channels
// 16 (w / 4) .. +15); warp 16 owns tensor memory and issues the MMAs. Operand stages are
// double-buffered, so a tile's branch sums overlap the previous tile's MMAs and drain. Every
// wait is a bounded mbarrier wait.
#include "chan_tc.cuh"
#include "ptx.cuh"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>

namespace rfx {

static __device__ unsigned int g_fault_chan_tc;

namespace {

constexpr int kM = 64;                 // channels
constexpr int kK = 2 * kM;             // GEMM K and N: Re and Im parts
constexpr int kFrames = 128;           // frames per tile = MMA M
constexpr int kR = 8;                  // frames per thread
constexpr int kWorkerWarps = 16;
constexpr int kMmaWarp = 16;
constexpr int kThreads = 17 * 32;
constexpr int kParts = 4;              // TMEM accumulators, 2 K-steps each
constexpr uint32_t kTmemCols = 512;    // kParts x kK
constexpr uint32_t kPlane = kFrames * 16 + 16;  // bytes per 8-element K plane (+16: banks)
constexpr uint32_t kSplit = (kK / 8) * kPlane;  // one split of one operand
constexpr uint32_t kIdesc = (1u << 4) | (static_cast<uint32_t>(kK >> 3) << 17) |
                            (static_cast<uint32_t>(kFrames >> 4) << 24);
constexpr int kWExp = 14;              // W' = 2^14 W, |W| <= 1

struct Layout {
    uint32_t w_hi, w_lo, a0, taps, bytes;
};

__host__ __device__ inline Layout chan_layout(int num_taps)
{
    Layout l;
    l.w_hi = 1024;
    l.w_lo = l.w_hi + kSplit;
    l.a0 = l.w_lo + kSplit;                       // two stages of (hi, lo)
    l.taps = l.a0 + 2 * 2 * kSplit;
    l.bytes = l.taps + ((4u * static_cast<uint32_t>(num_taps) + 15u) & ~15u);
    return l;
}

struct Ctrl {
    unsigned long long full[2];
    unsigned long long empty[2];
    unsigned long long dfull;
    unsigned long long dempty;
    unsigned long long reduce[2];
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
    uint32_t warp_max[2][kWorkerWarps];
};

__device__ __forceinline__ unsigned long long smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<unsigned long long>((addr >> 4) & 0x3FFFu) |
           (static_cast<unsigned long long>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<unsigned long long>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_f16(uint32_t d, unsigned long long a, unsigned long long b,
                                        uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ float exp2i(int e)
{
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}

__device__ __forceinline__ int scale_exponent(uint32_t abs_bits)
{
    return abs_bits == 0 ? 0 : 141 - static_cast<int>((abs_bits >> 23) & 0xFFu);
}

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

// s_d = x[(t0 + d) M - m] for d in [d0, d0 + 8): one 8-sample block of the decimated branch.
__device__ __forceinline__ void load_branch_block(f32x2 (&blk)[kR], const float2* __restrict__ x,
                                                  long long n, long long t0, int m, int d0)
{
#pragma unroll
    for (int i = 0; i < kR; ++i) {
        const long long s = (t0 + d0 + i) * kM - m;
        f32x2 v = 0ull;
        if (s >= 0 && s < n) {
            const float2 w = __ldg(x + s);
            v = pack2(w.x, w.y);
        }
        blk[i] = v;
    }
}

// Eight taps 8g + q (q < nq) of one branch: acc[i] += g_p s_{i - p}, cur = S_g, nxt = S_{g+1}
// where S_g[i] = s_{-8g + i}.
__device__ __forceinline__ void branch_group(f32x2 (&acc)[kR], const f32x2 (&cur)[kR],
                                             const f32x2 (&nxt)[kR], const float* taps_s, int m,
                                             int p0, int nq, int num_taps)
{
#pragma unroll
    for (int q = 0; q < kR; ++q) {
        if (q < nq) {
            const int l = (p0 + q) * kM + m;
            const float hv = l < num_taps ? taps_s[l] : 0.0f;
            const f32x2 h2 = pack2(hv, hv);
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                acc[i] = fma2(h2, i >= q ? cur[i - q] : nxt[kR + i - q], acc[i]);
            }
        }
    }
}

// u[t0 + i][m] for i < 8. Samples outside [0, n) read as zero; frames past the last one are
// computed on zeros and discarded by the caller.
__device__ __forceinline__ void branch_sums(f32x2 (&acc)[kR], const float2* __restrict__ x,
                                            long long n, const float* taps_s, long long t0,
                                            int m, int num_taps)
{
#pragma unroll
    for (int i = 0; i < kR; ++i) {
        acc[i] = 0ull;
    }
    const int per_branch = (num_taps + kM - 1) / kM;  // taps per branch P
    const int groups = per_branch / kR;
    const int rem = per_branch - groups * kR;
    f32x2 a[kR];
    f32x2 b[kR];
    load_branch_block(a, x, n, t0, m, 0);
    int g = 0;
    for (; g + 2 <= groups; g += 2) {
        load_branch_block(b, x, n, t0, m, -kR * (g + 1));
        branch_group(acc, a, b, taps_s, m, kR * g, kR, num_taps);
        load_branch_block(a, x, n, t0, m, -kR * (g + 2));
        branch_group(acc, b, a, taps_s, m, kR * (g + 1), kR, num_taps);
    }
    if (g < groups) {
        load_branch_block(b, x, n, t0, m, -kR * (g + 1));
        branch_group(acc, a, b, taps_s, m, kR * g, kR, num_taps);
        if (rem > 0) {
            load_branch_block(a, x, n, t0, m, -kR * (g + 2));
            branch_group(acc, b, a, taps_s, m, kR * (g + 1), rem, num_taps);
        }
    } else if (rem > 0) {
        load_branch_block(b, x, n, t0, m, -kR * (g + 1));
        branch_group(acc, a, b, taps_s, m, kR * g, rem, num_taps);
    }
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 1)
chan_tc_kernel(const float2* __restrict__ x, const float* __restrict__ taps,
               const uint16_t* __restrict__ w_img, float2* __restrict__ z, long long n,
               long long frames, int num_taps, int num_tiles)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const Layout lay = chan_layout(num_taps);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_chan_tc;
    const int my_tiles = static_cast<int>(blockIdx.x) < num_tiles
                             ? (num_tiles - 1 - static_cast<int>(blockIdx.x)) / gridDim.x + 1
                             : 0;
    float* taps_s = reinterpret_cast<float*>(smem + lay.taps);

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(smem_u32(&ctl.full[i]), kWorkerWarps);
            mbar_init(smem_u32(&ctl.empty[i]), 1);
            mbar_init(smem_u32(&ctl.reduce[i]), kWorkerWarps);
        }
        mbar_init(smem_u32(&ctl.dfull), 1);
        mbar_init(smem_u32(&ctl.dempty), kWorkerWarps);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&ctl.tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // The twiddle operand (hi and lo, already in the operand layout) and the taps.
    {
        const uint4* src = reinterpret_cast<const uint4*>(w_img);
        uint4* dst = reinterpret_cast<uint4*>(smem + lay.w_hi);
        for (uint32_t i = threadIdx.x; i < 2 * kSplit / 16; i += kThreads) {
            dst[i] = __ldg(src + i);
        }
        for (int k = threadIdx.x; k < num_taps; k += kThreads) {
            taps_s[k] = __ldg(taps + k);
        }
    }
    fence_proxy_async_smem();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = ctl.tmem_base;

    if (warp < kWorkerWarps) {
        const int wtid = threadIdx.x;
        // Branch-sum item of this thread: branches 2j, 2j+1, frames 8g .. 8g+7 of the tile.
        const int pair = wtid & 31;
        const int fgroup = wtid >> 5;
        const int quarter = warp & 3;
        const int slice = warp >> 2;                     // channels 16 slice .. +15
        int eu_ring[2] = {0, 0};

        auto produce = [&](int k) -> bool {
            const int tile = static_cast<int>(blockIdx.x) + k * gridDim.x;
            const long long t0 = static_cast<long long>(tile) * kFrames + kR * fgroup;
            f32x2 u0[kR];
            f32x2 u1[kR];
            branch_sums(u0, x, n, taps_s, t0, 2 * pair, num_taps);
            branch_sums(u1, x, n, taps_s, t0, 2 * pair + 1, num_taps);
            uint32_t mx = 0;
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                const float2 a = unpack2(u0[i]);
                const float2 b = unpack2(u1[i]);
                mx = max(mx, max(max(__float_as_uint(a.x) & 0x7FFFFFFFu,
                                     __float_as_uint(a.y) & 0x7FFFFFFFu),
                                 max(__float_as_uint(b.x) & 0x7FFFFFFFu,
                                     __float_as_uint(b.y) & 0x7FFFFFFFu)));
            }
            mx = __reduce_max_sync(0xFFFFFFFFu, mx);
            const int rb = k & 1;
            if (lane == 0) {
                ctl.warp_max[rb][warp] = mx;
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
            const int eu = scale_exponent(tmax);
            eu_ring[k & 1] = eu;
            const float fa = exp2i(eu / 2);
            const float fb = exp2i(eu - eu / 2);
            const int slot = k & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.empty[slot]), ((k >> 1) & 1) ^ 1, fault,
                                   kFaultStageEmpty, abort)) {
                return false;
            }
            // A operand: row = frame (8 fgroup + i), K = 2 pair (+1) for Re, 64 + 2 pair for Im.
            const uint32_t a_hi = sbase + lay.a0 + static_cast<uint32_t>(slot) * 2u * kSplit;
            const uint32_t a_lo = a_hi + kSplit;
            const int kre = 2 * pair;
            const int kim = kM + 2 * pair;
            const uint32_t off_re = static_cast<uint32_t>(kre >> 3) * kPlane + (kre & 7) * 2u;
            const uint32_t off_im = static_cast<uint32_t>(kim >> 3) * kPlane + (kim & 7) * 2u;
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                const float2 a = unpack2(u0[i]);
                const float2 b = unpack2(u1[i]);
                uint32_t re_hi, re_lo, im_hi, im_lo;
                split2(a.x * fa * fb, b.x * fa * fb, re_hi, re_lo);
                split2(a.y * fa * fb, b.y * fa * fb, im_hi, im_lo);
                const uint32_t row = static_cast<uint32_t>(kR * fgroup + i) * 16u;
                sts32(a_hi + off_re + row, re_hi);
                sts32(a_lo + off_re + row, re_lo);
                sts32(a_hi + off_im + row, im_hi);
                sts32(a_lo + off_im + row, im_lo);
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.full[slot]));
            }
            return true;
        };

        bool ok = true;
        for (int k = 0; k < 2 && k < my_tiles && ok; ++k) {
            ok = produce(k);
        }
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quarter * 32) << 16);
        for (int k = 0; k < my_tiles && ok && !*abort; ++k) {
            if (!mbar_wait_bounded(smem_u32(&ctl.dfull), k & 1, fault, kFaultAccumFull, abort)) {
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float re[16];
            float im[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                re[i] = 0.0f;
                im[i] = 0.0f;
            }
#pragma unroll
            for (int part = 0; part < kParts; ++part) {
                uint32_t tr[16];
                uint32_t ti[16];
                const uint32_t col = static_cast<uint32_t>(part * kK + 16 * slice);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(tr[0]), "=r"(tr[1]), "=r"(tr[2]), "=r"(tr[3]), "=r"(tr[4]),
                      "=r"(tr[5]), "=r"(tr[6]), "=r"(tr[7]), "=r"(tr[8]), "=r"(tr[9]),
                      "=r"(tr[10]), "=r"(tr[11]), "=r"(tr[12]), "=r"(tr[13]), "=r"(tr[14]),
                      "=r"(tr[15])
                    : "r"(lane_addr + col));
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(ti[0]), "=r"(ti[1]), "=r"(ti[2]), "=r"(ti[3]), "=r"(ti[4]),
                      "=r"(ti[5]), "=r"(ti[6]), "=r"(ti[7]), "=r"(ti[8]), "=r"(ti[9]),
                      "=r"(ti[10]), "=r"(ti[11]), "=r"(ti[12]), "=r"(ti[13]), "=r"(ti[14]),
                      "=r"(ti[15])
                    : "r"(lane_addr + col + kM));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    re[i] += __uint_as_float(tr[i]);
                    im[i] += __uint_as_float(ti[i]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.dempty));
            }
            const int shift = -(eu_ring[k & 1] + kWExp);
            const float fa = exp2i(shift / 2);
            const float fb = exp2i(shift - shift / 2);
            const int tile = static_cast<int>(blockIdx.x) + k * gridDim.x;
            const long long t = static_cast<long long>(tile) * kFrames + quarter * 32 + lane;
            if (t < frames) {
                float4* dst = reinterpret_cast<float4*>(z + t * kM + 16 * slice);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    dst[i] = make_float4(re[2 * i] * fa * fb, im[2 * i] * fa * fb,
                                         re[2 * i + 1] * fa * fb, im[2 * i + 1] * fa * fb);
                }
            }
            if (k + 2 < my_tiles) {
                ok = produce(k + 2);
            }
        }
    } else if (lane == 0) {
        const uint32_t w_hi = sbase + lay.w_hi;
        const uint32_t w_lo = sbase + lay.w_lo;
        for (int k = 0; k < my_tiles && !*abort; ++k) {
            const int slot = k & 1;
            if (!mbar_wait_bounded(smem_u32(&ctl.full[slot]), (k >> 1) & 1, fault,
                                   kFaultStageFull, abort) ||
                !mbar_wait_bounded(smem_u32(&ctl.dempty), (k & 1) ^ 1, fault, kFaultAccumEmpty,
                                   abort)) {
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_hi = sbase + lay.a0 + static_cast<uint32_t>(slot) * 2u * kSplit;
            const uint32_t a_lo = a_hi + kSplit;
            for (int ks = 0; ks < kK / 16; ++ks) {
                const uint32_t d = tmem + static_cast<uint32_t>((ks / (kK / 16 / kParts)) * kK);
                const uint32_t off = static_cast<uint32_t>(2 * ks) * kPlane;
                const unsigned long long ah = smem_desc(a_hi + off, kPlane, 128);
                const unsigned long long al = smem_desc(a_lo + off, kPlane, 128);
                const unsigned long long bh = smem_desc(w_hi + off, kPlane, 128);
                const unsigned long long bl = smem_desc(w_lo + off, kPlane, 128);
                mma_f16(d, ah, bh, (ks % (kK / 16 / kParts)) != 0 ? 1u : 0u);
                mma_f16(d, ah, bl, 1u);
                mma_f16(d, al, bh, 1u);
            }
            mma_commit(smem_u32(&ctl.dfull));
            mma_commit(smem_u32(&ctl.empty[slot]));
        }
        mma_commit(smem_u32(&ctl.teardown));
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == kMmaWarp) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols));
    }
}

// Builds the twiddle operand image in FP64: B row n (output column), K index k (input
// column), n, k < 128: rows 0-63 give Re z, rows 64-127 Im z; K 0-63 multiply Re u, 64-127
// Im u. Element value 2^14 W split into FP16 hi/lo, stored at the operand layout's offsets.
__global__ void chan_twiddle_kernel(uint16_t* img)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kK * kK) {
        return;
    }
    const int nrow = idx / kK;
    const int kcol = idx % kK;
    const int ch = nrow % kM;
    const int br = kcol % kM;
    double s, c;
    sincospi(2.0 * static_cast<double>((ch * br) % kM) / kM, &s, &c);
    double v;
    if (nrow < kM) {
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
    return channels == kM && num_taps >= 1 && chan_layout(num_taps).bytes <= 227u * 1024u;
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

cudaError_t chan_tc_launch(const void* x, const float* taps, const void* twiddles, void* z,
                           long long n, int num_taps, cudaStream_t stream)
{
    const long long frames = (n + kM - 1) / kM;
    if (frames == 0) {
        return cudaSuccess;
    }
    const Layout lay = chan_layout(num_taps);
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    const uint32_t bytes = lay.bytes > 120u * 1024u ? lay.bytes : 120u * 1024u;
    // The block's warps must fit the register file at this register count.
    cudaFuncAttributes attr{};
    if ((err = cudaFuncGetAttributes(&attr, chan_tc_kernel)) != cudaSuccess) {
        return err;
    }
    if (attr.maxThreadsPerBlock < kThreads) {
        return cudaErrorLaunchOutOfResources;
    }
    err = cudaFuncSetAttribute(chan_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(bytes));
    if (err != cudaSuccess) {
        return err;
    }
    const int tiles = static_cast<int>((frames + kFrames - 1) / kFrames);
    const int grid = tiles < sms ? tiles : sms;
    chan_tc_kernel<<<grid, kThreads, bytes, stream>>>(
        static_cast<const float2*>(x), taps, static_cast<const uint16_t*>(twiddles),
        static_cast<float2*>(z), n, frames, num_taps, tiles);
    return cudaGetLastError();
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
