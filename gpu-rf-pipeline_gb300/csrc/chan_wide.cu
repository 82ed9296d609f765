// Tensor-core 1024-point DFT of the 1024-channel polyphase channelizer, sm_103a.
//
//   u[t][m] = sum_p h[pM + m] x[tM - pM - m]   (x[i < 0] = 0)     src/channelize.cu:25-49
//   z[t][k] = sum_m u[t][m] e^{+2 pi i k m / M}, M = 1024           src/channelize.cu:70-71
//
// The branch sums u come from chan_branch_launch (csrc/chan_plain.cu: the reference's FP32
// arithmetic, bit for bit; the register-ring kernel for 8 to 32 taps per branch). This file
// computes the DFT, factored 32 x 32 (m = m1 + 32 m2, k = k2 + 32 k1, w_N = e^{+2 pi i/N}):
//   A[m1][k2]     = sum_m2 u[m1 + 32 m2] w_32^(k2 m2)        stage 1, a complex GEMM
//   B[m1][k2]     = A[m1][k2] w_1024^(k2 m1)                  twiddle, FP32
//   z[k2 + 32 k1] = sum_m1 B[m1][k2] w_32^(k1 m1)             stage 2, a complex GEMM
// Both GEMMs run on tcgen05 (M = 128, N = 64, K = 64 real) against the same matrix
// W = 2^14 [[cos, sin], [-sin, cos]](2 pi k m / 32) (K rows: Re in, Im in; N columns: Re out,
// Im out), built in FP64 and split into FP16 hi + lo once. Each operand is split the same way
// after a power-of-two scale per frame, and three split products accumulate in FP32 (twelve
// MMAs per accumulator, well inside the round-toward-zero accumulation's error budget).
//
// A CTA takes groups of 4 frames (4 x 32 = 128 GEMM rows) in turn; warp q (0-3) handles frame
// q of each group, i.e. TMEM lanes 32 q .. 32 q + 31, and warp 4 issues the MMAs:
//  1. lane m1 reads u[m1 + 32 m2], m2 = 0..31, from the group's buffer (warp 5 brings each group's
//     32 contiguous KB in with one bulk copy, a group ahead); the frame's largest
//     component sets its scale 2^e1; the split values are stage 1's A operand, row 32 q + m1
//     (K-major).
//  2. Stage 1 into TMEM columns 0-63.
//  3. Lane m1 loads its row (Re, Im of k2 = 0..31), undoes 2^(e1 + 14), multiplies the twiddle
//     w_1024^(k2 m1), scales by 2^e2 = 2^(e1 - 6) and writes stage 2's A operand MN-major (row
//     32 q + k2, K index m1): a thread's values for one K index are consecutive rows, so each
//     store is 16 contiguous bytes.
//  4. Stage 2 (A MN-major) into columns 64-127.
//  5. Lane k2 loads its row (Re, Im of k1 = 0..31), undoes 2^(e2 + 14) and stores channels
//     k2 + 32 k1 (a warp's store is 256 contiguous bytes), or their magnitudes.
// A group's steps are a chain of dependent waits; two CTAs share an SM (112 KB of shared
// memory and 128 TMEM columns each) and interleave their groups. Measured at 2^16 frames: 244 us
// per launch (DRAM 52 %, tensor pipe 18 %), and within 1 % of that with u loaded straight into
// registers (four CTAs an SM), two warps per frame, padded operand planes, or one accumulator
// per split product; with the MMAs left out (a timing copy) the branch + DFT step still took
// 418 us against 455 us, so the MMAs are not what bounds it either.
//
// Measured and not kept: one fused kernel on clusters of four CTAs (each CTA computing the
// branch sums of 256 branches and the DFT of every fourth frame group, the sums exchanged
// through L2 or distributed shared memory) ran 590-690 us at 2^26 samples, against 355 us for
// branch sums + cuFFT: its single set of four DFT warps per SM spent about 11000 cycles per
// group in that chain, and every branch warp waited on them.
#include "chan_plain.cuh"
#include "chan_wide.cuh"
#include "magnitude.cuh"
#include "tc_common.cuh"

#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_chan_wide;

namespace {

using namespace tc;

constexpr int kM = 1024;
constexpr int kRadix = 32;
constexpr int kGroup = 4;                    // frames per group (4 x 32 rows = MMA M)
constexpr int kMmaWarp = 4;
constexpr int kLoadWarp = 5;
constexpr int kThreads = 6 * 32;
constexpr int kK = 2 * kRadix;               // GEMM K and N: Re and Im parts
constexpr uint32_t kIdesc1 = idesc_f16(128, kK);
constexpr uint32_t kIdesc2 = idesc_f16(128, kK) | (1u << 15);   // A MN-major
constexpr int kWExp = 14;
constexpr uint32_t kTmemCols = 128;
constexpr unsigned kFull = 0xFFFFFFFFu;

// Shared memory (bytes from the 1024-aligned base): control block, W hi and lo (copied from
// the plan's image), the A operand hi and lo, two group buffers of u: 112 KB, two CTAs an SM.
constexpr uint32_t kWPlane = kK * 16;                   // one 8-element K group of W (64 rows)
constexpr uint32_t kWSplit = 8 * kWPlane;
constexpr uint32_t kAPlane = 128 * 16;                  // one 8-element K group of A (128 rows)
constexpr uint32_t kASplit = 8 * kAPlane;
constexpr uint32_t kOffW = 128;
constexpr uint32_t kImageBytes = 2 * kWSplit + kRadix * kRadix * 8;   // W hi, W lo, twiddles
constexpr uint32_t kOffA = kOffW + 2 * kWSplit;
constexpr uint32_t kOffU = kOffA + 2 * kASplit;
constexpr uint32_t kUBytes = kGroup * kM * 8;           // one group of u: 32 KB, contiguous
constexpr uint32_t kSmemBytes = kOffU + 2 * kUBytes;

struct Ctrl {
    unsigned long long u_full[2];         // a group's u has landed (bulk copy, bytes)
    unsigned long long u_empty[2];        // the DFT warps have read it (4 warps)
    unsigned long long a_full;            // operand written (4 DFT warps): A1, A2, A1, ...
    unsigned long long d1_full;           // stage-1 accumulator complete (MMA commit)
    unsigned long long d2_full;           // stage-2 accumulator complete
    unsigned long long teardown;
    uint32_t tmem_base;
    int abort;
};
static_assert(sizeof(Ctrl) <= kOffW, "control block");

__device__ __forceinline__ void sts128(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                       uint32_t d)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c),
                 "r"(d)
                 : "memory");
}

// Lane 0 waits, the warp synchronizes behind it, and every lane gets lane 0's result: the warp
// never splits at a later warp-wide step.
__device__ __forceinline__ bool lead_wait(uint32_t bar, uint32_t parity, unsigned int* fault,
                                          unsigned int code, volatile int* abort)
{
    bool ok = true;
    if ((threadIdx.x & 31) == 0) {
        ok = mbar_wait_bounded(bar, parity, fault, code, abort);
    }
    __syncwarp();
    return __shfl_sync(kFull, ok ? 1 : 0, 0) != 0;
}

}  // namespace

template <bool kMag>
__global__ void __launch_bounds__(kThreads, 2)
chan_dft_kernel(const float2* __restrict__ u, const uint4* __restrict__ image,
                void* __restrict__ out, long long frames, long long groups)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    Ctrl& ctl = *reinterpret_cast<Ctrl*>(smem);
    const int warp = static_cast<int>(threadIdx.x >> 5);
    const int lane = static_cast<int>(threadIdx.x & 31);
    const uint32_t sbase = smem_u32(smem);
    volatile int* abort = &ctl.abort;
    unsigned int* fault = &g_fault_chan_wide;

    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&ctl.u_full[b]), 1);
            mbar_init(smem_u32(&ctl.u_empty[b]), 4);
        }
        mbar_init(smem_u32(&ctl.a_full), 4);
        mbar_init(smem_u32(&ctl.d1_full), 1);
        mbar_init(smem_u32(&ctl.d2_full), 1);
        mbar_init(smem_u32(&ctl.teardown), 1);
        ctl.abort = 0;
        fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tmem_alloc(smem_u32(&ctl.tmem_base), kTmemCols);
    }
    {
        uint4* dst = reinterpret_cast<uint4*>(smem + kOffW);
        for (uint32_t i = threadIdx.x; i < 2 * kWSplit / 16; i += kThreads) {
            dst[i] = __ldg(image + i);
        }
    }
    fence_proxy_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;
    const long long g0 = blockIdx.x;
    const long long gstep = gridDim.x;

    if (warp < kMmaWarp) {
        const int q = warp;                          // frame of each group; TMEM lanes 32 q ..
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(q * 32) << 16);
        const uint32_t a_hi = sbase + kOffA;
        const uint32_t a_lo = a_hi + kASplit;
        // Stage 1 A: row 32 q + lane, K groups 0-3 = Re of m2 = 8 g .. + 7, 4-7 = Im.
        const uint32_t row1 = static_cast<uint32_t>(q * 4 + (lane >> 3)) * 128u +
                              static_cast<uint32_t>(lane & 7) * 16u;
        // Stage 2 A (MN-major): K index lane (Re) / 32 + lane (Im) = K group lane / 8 (+ 4),
        // row lane % 8 of the core matrices; rows 32 q + 8 i .. + 7 = MN block 4 q + i.
        const uint32_t k2re = static_cast<uint32_t>(lane >> 3) * kAPlane +
                              static_cast<uint32_t>(lane & 7) * 16u +
                              static_cast<uint32_t>(q * 4) * 128u;
        const uint32_t k2im = k2re + 4 * kAPlane;
        // tw[k2][lane] = w_1024^(k2 lane): the plan image's table, read through L1.
        const float2* tw = reinterpret_cast<const float2*>(image + 2 * kWSplit / 16) + lane;
        float2 v[kRadix];
        long long jj = 0;
        for (long long g = g0; g < groups; g += gstep, ++jj) {
            if (__any_sync(kFull, *abort != 0)) {
                break;
            }
            // u[m1 + 32 m2] of frame q from the group's buffer (a warp's loads of one m2 are
            // 256 contiguous bytes), which then goes back to the load warp.
            const uint32_t b = static_cast<uint32_t>(jj & 1);
            if (!lead_wait(smem_u32(&ctl.u_full[b]), static_cast<uint32_t>((jj >> 1) & 1), fault,
                           kFaultTileLoad, abort)) {
                break;
            }
            {
                const uint32_t src = sbase + kOffU + b * kUBytes +
                                     static_cast<uint32_t>(q * kM * 8 + lane * 8);
#pragma unroll
                for (int m2 = 0; m2 < kRadix; ++m2) {
                    v[m2] = unpack2(lds64(src + static_cast<uint32_t>(m2 * kRadix * 8)));
                }
            }
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.u_empty[b]));
            }
            // 1. Stage 1's operand: frame q, scaled by 2^e1.
            uint32_t mx = 0;
#pragma unroll
            for (int m2 = 0; m2 < kRadix; ++m2) {
                mx = max(mx, max(absbits(v[m2].x), absbits(v[m2].y)));
            }
            const int e1 = min(scale_exponent(__reduce_max_sync(kFull, mx)), 127);
            {
                const float fs = exp2_exact(e1);
                const f32x2 f = pack2(fs, fs);
#pragma unroll
                for (int gk = 0; gk < 4; ++gk) {
                    uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 p0 = unpack2(mul2(pack2(v[8 * gk + 2 * e].x,
                                                             v[8 * gk + 2 * e].y), f));
                        const float2 p1 = unpack2(mul2(pack2(v[8 * gk + 2 * e + 1].x,
                                                             v[8 * gk + 2 * e + 1].y), f));
                        split2(p0.x, p1.x, rh[e], rl[e]);
                        split2(p0.y, p1.y, ih[e], il[e]);
                    }
                    const uint32_t gre = static_cast<uint32_t>(gk) * kAPlane + row1;
                    const uint32_t gim = static_cast<uint32_t>(gk + 4) * kAPlane + row1;
                    sts128(a_hi + gre, rh[0], rh[1], rh[2], rh[3]);
                    sts128(a_lo + gre, rl[0], rl[1], rl[2], rl[3]);
                    sts128(a_hi + gim, ih[0], ih[1], ih[2], ih[3]);
                    sts128(a_lo + gim, il[0], il[1], il[2], il[3]);
                }
            }
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.a_full));
            }
            // 3. Stage 1's row m1 = lane: Re (columns 0-31) and Im (32-63) of k2.
            if (!lead_wait(smem_u32(&ctl.d1_full), static_cast<uint32_t>(jj & 1), fault,
                           kFaultAccumFull, abort)) {
                break;
            }
            fence_after();
            // B = A w_1024^(k2 m1) has modulus at most 32 max|u| < 2^(6 - e1) 2^15 (a sum of 32
            // terms of modulus < 2^15.5 2^-e1, and |w| = 1), so the frame's stage-2 scale 2^e2,
            // e2 = e1 - 6, keeps every component below 2^15 without another pass for the largest;
            // the FP16 hi/lo split has the same relative precision at any power-of-two scale.
            const int e2 = e1 - 6;
            {
                const float s1 = exp2_exact(-(e1 + kWExp));
                const float f = exp2_exact(e2);
#pragma unroll
                for (int part = 0; part < 4; ++part) {     // k2 = 8 part .. + 7: MN block 4 q + part
                    uint32_t tre[8];
                    uint32_t tim[8];
                    tmem_ld8(lane_addr + static_cast<uint32_t>(8 * part), tre);
                    tmem_ld8(lane_addr + static_cast<uint32_t>(kRadix + 8 * part), tim);
                    tmem_wait_ld();
                    uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        float2 b[2];
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            const int i = 2 * e + j;
                            const float re = __uint_as_float(tre[i]) * s1;
                            const float im = __uint_as_float(tim[i]) * s1;
                            const float2 w = __ldg(tw + (8 * part + i) * kRadix);
                            b[j] = make_float2((re * w.x - im * w.y) * f, (re * w.y + im * w.x) * f);
                        }
                        split2(b[0].x, b[1].x, rh[e], rl[e]);
                        split2(b[0].y, b[1].y, ih[e], il[e]);
                    }
                    const uint32_t blk = static_cast<uint32_t>(part) * 128u;
                    sts128(a_hi + k2re + blk, rh[0], rh[1], rh[2], rh[3]);
                    sts128(a_lo + k2re + blk, rl[0], rl[1], rl[2], rl[3]);
                    sts128(a_hi + k2im + blk, ih[0], ih[1], ih[2], ih[3]);
                    sts128(a_lo + k2im + blk, il[0], il[1], il[2], il[3]);
                }
            }
            fence_before();
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(smem_u32(&ctl.a_full));
            }
            // 5. Stage 2's row k2 = lane: Re (columns 64-95) and Im (96-127) of k1.
            if (!lead_wait(smem_u32(&ctl.d2_full), static_cast<uint32_t>(jj & 1), fault,
                           kFaultAccumFull, abort)) {
                break;
            }
            fence_after();
            const float s2 = exp2_exact(-(e2 + kWExp));
            const long long t = kGroup * g + q;
#pragma unroll
            for (int part = 0; part < 4; ++part) {
                uint32_t tre[8];
                uint32_t tim[8];
                tmem_ld8(lane_addr + static_cast<uint32_t>(2 * kRadix + 8 * part), tre);
                tmem_ld8(lane_addr + static_cast<uint32_t>(3 * kRadix + 8 * part), tim);
                tmem_wait_ld();
                if (t < frames) {
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int k1 = 8 * part + i;
                        const float re = __uint_as_float(tre[i]) * s2;
                        const float im = __uint_as_float(tim[i]) * s2;
                        const long long o = t * kM + lane + kRadix * k1;
                        if constexpr (kMag) {
                            __stcs(static_cast<float*>(out) + o, cmag(re, im));
                        } else {
                            __stcs(static_cast<float2*>(out) + o, make_float2(re, im));
                        }
                    }
                }
            }
            fence_before();
        }
    } else if (warp == kMmaWarp && lane == 0) {
        const uint32_t a_hi = sbase + kOffA;
        const uint32_t a_lo = a_hi + kASplit;
        const uint32_t w_hi = sbase + kOffW;
        const uint32_t w_lo = w_hi + kWSplit;
        for (long long g = g0; g < groups && !*abort; g += gstep) {
            for (int stage = 0; stage < 2; ++stage) {
                if (!mbar_wait_bounded(smem_u32(&ctl.a_full), static_cast<uint32_t>(stage), fault,
                                       kFaultStageFull, abort)) {
                    break;
                }
                fence_after();
                const uint32_t d = tmem + static_cast<uint32_t>(stage * kK);
#pragma unroll
                for (int ks = 0; ks < kK / 16; ++ks) {
                    const uint32_t aoff = static_cast<uint32_t>(2 * ks) * kAPlane;
                    const uint32_t woff = static_cast<uint32_t>(2 * ks) * kWPlane;
                    const unsigned long long ah = smem_desc(a_hi + aoff, kAPlane, 128);
                    const unsigned long long al = smem_desc(a_lo + aoff, kAPlane, 128);
                    const unsigned long long bh = smem_desc(w_hi + woff, kWPlane, 128);
                    const unsigned long long bl = smem_desc(w_lo + woff, kWPlane, 128);
                    if (stage == 0) {
                        mma_f16<kIdesc1>(d, ah, bh, ks != 0 ? 1u : 0u);
                        mma_f16<kIdesc1>(d, ah, bl, 1u);
                        mma_f16<kIdesc1>(d, al, bh, 1u);
                    } else {
                        mma_f16<kIdesc2>(d, ah, bh, ks != 0 ? 1u : 0u);
                        mma_f16<kIdesc2>(d, ah, bl, 1u);
                        mma_f16<kIdesc2>(d, al, bh, 1u);
                    }
                }
                mma_commit(smem_u32(stage == 0 ? &ctl.d1_full : &ctl.d2_full));
            }
        }
        mma_commit(smem_u32(&ctl.teardown));
        mbar_wait_bounded(smem_u32(&ctl.teardown), 0, fault, kFaultTeardown, nullptr);
    } else if (warp == kLoadWarp && lane == 0) {
        // Each group's u (4 consecutive frames: one contiguous 32 KB stretch, fewer bytes for
        // the last group) by one bulk copy into buffer jj % 2, one group ahead of the DFT warps.
        long long jj = 0;
        for (long long g = g0; g < groups && !*abort; g += gstep, ++jj) {
            const uint32_t b = static_cast<uint32_t>(jj & 1);
            if (!mbar_wait_bounded(smem_u32(&ctl.u_empty[b]),
                                   static_cast<uint32_t>(((jj >> 1) & 1) ^ 1), fault,
                                   kFaultStageEmpty, abort)) {
                break;
            }
            const long long left = frames - kGroup * g;
            const uint32_t bytes = static_cast<uint32_t>(left < kGroup ? left : kGroup) * kM * 8u;
            const uint32_t bar = smem_u32(&ctl.u_full[b]);
            mbar_arrive_expect_tx(bar, bytes);
            bulk_g2s(sbase + kOffU + b * kUBytes, u + kGroup * g * kM, bytes, bar);
        }
        // No copy may still be writing this CTA's shared memory when it exits (after an abort
        // the DFT warps may not have waited for the last ones).
        for (long long i = jj - 2 > 0 ? jj - 2 : 0; i < jj; ++i) {
            mbar_wait_bounded(smem_u32(&ctl.u_full[i & 1]), static_cast<uint32_t>((i >> 1) & 1),
                              fault, kFaultTileLoad, nullptr);
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == kMmaWarp) {
        tmem_dealloc(tmem, kTmemCols);
    }
}

// The plan's image: W hi and W lo in the B operand layout (K-major, 64 rows n x 64 K), then
// the twiddles w_1024^(k2 m1) as float2 at [k2][m1]; all from FP64 sin/cos.
__global__ void chan_wide_image_kernel(uint16_t* w_img, float2* tw)
{
    const int idx = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (idx < kK * kK) {
        const int n = idx / kK;      // output column: Re (n < 32) or Im of k_out = n % 32
        const int kk = idx % kK;     // K index: Re (kk < 32) or Im of m_in = kk % 32
        const int kout = n % kRadix;
        const int min_ = kk % kRadix;
        double s, c;
        sincospi(2.0 * static_cast<double>((kout * min_) % kRadix) / kRadix, &s, &c);
        double v;
        if (n < kRadix) {
            v = kk < kRadix ? c : -s;   // Re out = Re in cos - Im in sin
        } else {
            v = kk < kRadix ? s : c;    // Im out = Re in sin + Im in cos
        }
        const float vs = static_cast<float>(v * 16384.0);
        const __half hi = __float2half_rn(vs);
        const __half lo = __float2half_rn(vs - __half2float(hi));
        const uint32_t off = static_cast<uint32_t>(kk >> 3) * kWPlane +
                             static_cast<uint32_t>(n) * 16u + static_cast<uint32_t>(kk & 7) * 2u;
        w_img[off / 2] = *reinterpret_cast<const uint16_t*>(&hi);
        w_img[(kWSplit + off) / 2] = *reinterpret_cast<const uint16_t*>(&lo);
    }
    if (idx < kRadix * kRadix) {
        const int k2 = idx / kRadix;
        const int m1 = idx % kRadix;
        double s, c;
        sincospi(2.0 * static_cast<double>(k2 * m1) / kM, &s, &c);
        tw[idx] = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
}

bool chan_wide_supported(int channels) { return channels == kM; }

size_t chan_wide_image_bytes() { return kImageBytes; }

cudaError_t chan_wide_build_image(void* img, cudaStream_t stream)
{
    cudaError_t err = cudaMemsetAsync(img, 0, kImageBytes, stream);
    if (err != cudaSuccess) {
        return err;
    }
    chan_wide_image_kernel<<<(kK * kK + 255) / 256, 256, 0, stream>>>(
        static_cast<uint16_t*>(img),
        reinterpret_cast<float2*>(static_cast<unsigned char*>(img) + 2 * kWSplit));
    return cudaGetLastError();
}

template <bool kMag>
static cudaError_t launch_dft(const float2* u, const void* image, void* z, long long frames,
                              cudaStream_t stream)
{
    auto kernel = chan_dft_kernel<kMag>;
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess ||
        (err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(kSmemBytes))) != cudaSuccess ||
        (err = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    cudaSharedmemCarveoutMaxShared)) != cudaSuccess) {
        return err;
    }
    // Persistent CTAs, two per SM (shared memory), each taking every grid-th group.
    constexpr int occ = 2;
    const long long groups = (frames + kGroup - 1) / kGroup;
    const long long cap = static_cast<long long>(sms) * occ;
    const unsigned grid = static_cast<unsigned>(groups < cap ? groups : cap);
    kernel<<<grid, kThreads, kSmemBytes, stream>>>(u, static_cast<const uint4*>(image), z, frames,
                                                   groups);
    return cudaGetLastError();
}

cudaError_t chan_wide_launch(const void* x, const float* taps, const void* image, void* u,
                             void* z, long long n, int num_taps, cudaStream_t stream,
                             bool magnitude, int format)
{
    const long long frames = (n + kM - 1) / kM;
    if (frames == 0) {
        return cudaSuccess;
    }
    cudaError_t err = chan_branch_launch(x, taps, u, frames, kM, num_taps, stream, format);
    if (err != cudaSuccess) {
        return err;
    }
    const float2* uf = static_cast<const float2*>(u);
    return magnitude ? launch_dft<true>(uf, image, z, frames, stream)
                     : launch_dft<false>(uf, image, z, frames, stream);
}

cudaError_t chan_wide_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_chan_wide, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_chan_wide, &zero, sizeof(unsigned int));
}

}  // namespace rfx
