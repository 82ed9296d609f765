// The plain FP32 FIR's tile function (one tile of 2304 outputs computed by a group of 256
// threads), shared by the plain kernels (fir_plain.cu) and the persistent batch kernel
// (fir_batch.cu), which runs plain tiles with groups of its own threads.
//
//   y[n] = sum_{k=0}^{K-1} h[k] x[n-k],  x[m] = 0 for m < 0,  n < N      (src/fir.cu:1-5)
//
// Arithmetic: every output is one chain of fused multiply-adds over k = 0, 1, ..., K-1 starting
// from +0.0f, separately for I and Q. That is the order of the project's naive, tiled and
// register kernels (src/fir.cu:35-40, :377-395), so the results are bit-identical to theirs.
// Taps past the start of the input multiply zeros, which leaves the chain unchanged.
//
// Work decomposition: a group of 256 threads owns a tile of 2304 consecutive outputs; thread t
// owns outputs t0 + 9t ... t0 + 9t + 8. Nine (odd) outputs per thread put the 64-bit shared
// loads of a warp (stride 72 bytes) on distinct bank pairs.
//
// Staging: the tile's samples x[t0 - (K-1) .. t0 + 2303] (start rounded down to an even index so
// the copy is 16-byte aligned) arrive in shared memory through ONE bulk copy on the TMA engine,
// completed on an mbarrier; tiles that touch either end of the input are filled by the threads
// with zeros outside [0, N). Results go back through shared memory and one bulk store.
//
// Inner loop: taps are taken nine at a time. For taps 9g .. 9g+8 a thread needs the 17 samples
// x[n0 - 9g - 8 .. n0 - 9g + 8] (n0 = its first output), i.e. the sample blocks
// S_g = x[n0 - 9g .. +8] and S_{g+1}. Two register blocks alternate between those roles, so
// sliding the window costs nine 64-bit loads per nine taps and no register moves. Each
// tap-sample product is one packed fma.rn.f32x2 on (I, Q) with the tap duplicated in both lanes.
#pragma once

#include "fir_plain.cuh"
#include "ptx.cuh"

#include <cuda_runtime.h>

namespace rfx {

// How the 256 threads of a tile synchronize: the whole block (the plain kernels), or one named
// barrier per group of 256 threads (the batch kernel's groups).
struct PlainBlockSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct PlainGroupSync {
    uint32_t id;
    __device__ __forceinline__ void operator()() const
    {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(kPlainThreads) : "memory");
    }
};

namespace plain {

constexpr int kThreads = kPlainThreads;
constexpr int kR = kPlainOutputsPerThread;
constexpr int kTile = kPlainTileOutputs;
constexpr int kGuard = 16;  // zero samples in front of the tile: the last window block may
                            // reach up to 10 samples before it (those values are never used)

struct Layout {
    uint32_t taps_off;   // (h, h) pairs, K entries
    uint32_t tile_off;   // guard + tile samples
    uint32_t raw_off;    // integer input formats: the tile's raw components as copied
    uint32_t bytes;
};

// Bytes per sample of each input format (rfx_sample_format): cf32, ci16, ci8.
__host__ __device__ constexpr uint32_t sample_bytes(int fmt) { return fmt == 0 ? 8u : fmt == 1 ? 4u : 2u; }

__host__ __device__ inline Layout plain_layout(int num_taps, int fmt = 0)
{
    Layout l;
    l.taps_off = 16;
    l.tile_off = (l.taps_off + 8u * static_cast<uint32_t>(num_taps) + 15u) & ~15u;
    const uint32_t tile_samples = kGuard + kTile + static_cast<uint32_t>(num_taps) + 8u;
    l.raw_off = (l.tile_off + 8u * tile_samples + 15u) & ~15u;
    l.bytes = l.raw_off + (fmt == 0 ? 0u : sample_bytes(fmt) * (kTile + static_cast<uint32_t>(num_taps) + 8u));
    return l;
}

// Sample i of an integer-format input, decoded as the project's SigMF reader does
// (src/io.cpp:110-124): component x (1/32768) for ci16_le, x (1/128) for ci8.
template <int kFmt>
__device__ __forceinline__ f32x2 decode_sample(const void* raw, long long i)
{
    if (kFmt == 1) {
        const short2 v = static_cast<const short2*>(raw)[i];
        return pack2(static_cast<float>(v.x) * (1.0f / 32768.0f),
                     static_cast<float>(v.y) * (1.0f / 32768.0f));
    }
    const char2 v = static_cast<const char2*>(raw)[i];
    return pack2(static_cast<float>(v.x) * (1.0f / 128.0f), static_cast<float>(v.y) * (1.0f / 128.0f));
}

// Nine taps 9g + q (q < nq) against output window blocks: cur = S_g, nxt = S_{g+1}.
__device__ __forceinline__ void tap_group(f32x2 (&acc)[kR], const f32x2 (&cur)[kR],
                                          const f32x2 (&nxt)[kR], const f32x2* taps2, int k0,
                                          int nq)
{
#pragma unroll
    for (int q = 0; q < kR; ++q) {
        if (q < nq) {
            const f32x2 h = taps2[k0 + q];
#pragma unroll
            for (int j = 0; j < kR; ++j) {
                acc[j] = fma2(h, j >= q ? cur[j - q] : nxt[kR + j - q], acc[j]);
            }
        }
    }
}

__device__ __forceinline__ void load_block(f32x2 (&blk)[kR], const f32x2* tile, int p, int m)
{
    // S_m[i] = x[n0 - 9m + i] = tile[p - 9m + i]
    const f32x2* src = tile + (p - kR * m);
#pragma unroll
    for (int i = 0; i < kR; ++i) {
        blk[i] = src[i];
    }
}

// Computes this thread's nine outputs of the tile staged at `tile` (tile[i] = x[base + i]).
__device__ __forceinline__ void compute_outputs(f32x2 (&acc)[kR], const f32x2* tile,
                                                const f32x2* taps2, int p, int num_taps)
{
#pragma unroll
    for (int j = 0; j < kR; ++j) {
        acc[j] = 0ull;  // +0.0f, +0.0f
    }
    const int groups = num_taps / kR;
    const int rem = num_taps - groups * kR;
    f32x2 a[kR];
    f32x2 b[kR];
    load_block(a, tile, p, 0);
    int g = 0;
    for (; g + 2 <= groups; g += 2) {
        load_block(b, tile, p, g + 1);
        tap_group(acc, a, b, taps2, kR * g, kR);
        load_block(a, tile, p, g + 2);
        tap_group(acc, b, a, taps2, kR * (g + 1), kR);
    }
    if (g < groups) {
        load_block(b, tile, p, g + 1);
        tap_group(acc, a, b, taps2, kR * g, kR);
        if (rem > 0) {
            load_block(a, tile, p, g + 2);
            tap_group(acc, b, a, taps2, kR * (g + 1), rem);
        }
    } else if (rem > 0) {
        load_block(b, tile, p, g + 1);
        tap_group(acc, a, b, taps2, kR * g, rem);
    }
}

}  // namespace plain

// One tile of one capture, computed by the 256 threads tid = 0..255 of a group that synchronizes
// with `sync`; the tile's mbarrier sits at smem offset 0 (initialized by this call if `init`,
// its expected phase in `phase`, advanced when the tile used it). Returns false if the tile's
// copy did not arrive within the wait limit (recorded in *fault). kFmt: the input's sample
// format (0 cf32; 1 ci16, 2 ci8: decoded into cf32 in shared memory).
template <int kFmt = 0, class Sync = PlainBlockSync>
__device__ __forceinline__ bool fir_plain_tile(const void* __restrict__ xv,
                                               const float* __restrict__ taps,
                                               float2* __restrict__ y, long long n,
                                               int num_taps, long long tile_index,
                                               unsigned char* smem, unsigned int* fault,
                                               int tid, Sync sync, uint32_t& phase, bool init)
{
    using namespace plain;
    const float2* x = static_cast<const float2*>(xv);
    const Layout lay = plain_layout(num_taps, kFmt);
    const uint32_t sbase = smem_u32(smem);
    const uint32_t bar = sbase;  // mbarrier at offset 0
    f32x2* taps2 = reinterpret_cast<f32x2*>(smem + lay.taps_off);
    f32x2* guard = reinterpret_cast<f32x2*>(smem + lay.tile_off);
    f32x2* tile = guard + kGuard;

    const long long t0 = tile_index * kTile;
    // First staged sample: a multiple of 2 (cf32) or 8 (integer formats) so that the copy
    // starts on a 16-byte boundary; the length is then a multiple of 16 bytes too.
    const long long base = (t0 - (num_taps - 1)) & (kFmt == 0 ? ~1ll : ~7ll);
    const int tile_len = static_cast<int>(t0 + kTile - base);
    const bool interior = base >= 0 && t0 + kTile <= n;

    if (init && tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    sync();
    if (interior && tid == 0) {
        const uint32_t bytes = sample_bytes(kFmt) * static_cast<uint32_t>(tile_len);
        mbar_arrive_expect_tx(bar, bytes);
        if (kFmt == 0) {
            bulk_g2s(smem_u32(tile), x + base, bytes, bar);
        } else {
            bulk_g2s(sbase + lay.raw_off,
                     static_cast<const unsigned char*>(xv) + sample_bytes(kFmt) * base, bytes, bar);
        }
    }
    // Taps (duplicated into both lanes) and the guard while the copy is in flight.
    for (int k = tid; k < num_taps; k += kThreads) {
        const float h = __ldg(taps + k);
        taps2[k] = pack2(h, h);
    }
    if (tid < kGuard) {
        guard[tid] = 0ull;
    }
    if (!interior) {
        for (int i = tid; i < tile_len; i += kThreads) {
            const long long m = base + i;
            f32x2 v = 0ull;
            if (m >= 0 && m < n) {
                if (kFmt == 0) {
                    const float2 s = x[m];
                    v = pack2(s.x, s.y);
                } else {
                    v = decode_sample<kFmt>(xv, m);
                }
            }
            tile[i] = v;
        }
    }
    sync();
    bool ok = true;
    if (interior) {
        ok = mbar_wait_bounded(bar, phase, fault, kFaultTileLoad, nullptr);
        phase ^= 1u;
        if (kFmt != 0) {
            // Decode the staged components into the sample tile.
            const unsigned char* raw = smem + lay.raw_off;
            for (int i = tid; i < tile_len; i += kThreads) {
                tile[i] = decode_sample<kFmt>(raw, i);
            }
            sync();
        }
    }

    const long long n0 = t0 + static_cast<long long>(kR) * tid;
    f32x2 acc[kR];
    if (ok && n0 < n) {
        compute_outputs(acc, tile, taps2, static_cast<int>(n0 - base), num_taps);
    }
    sync();  // every thread is done reading the tile: reuse it for the results
    if (ok && n0 < n) {
#pragma unroll
        for (int j = 0; j < kR; ++j) {
            tile[kR * tid + j] = acc[j];
        }
    }
    if (interior) {
        fence_proxy_async_smem();
    }
    sync();
    if (!ok) {
        return false;
    }
    if (interior) {
        if (tid == 0) {
            bulk_s2g(y + t0, smem_u32(tile), 8u * kTile);
            bulk_commit();
            bulk_wait_read_all();
        }
    } else {
        const long long valid = n - t0 < kTile ? n - t0 : kTile;
        for (int i = tid; i < valid; i += kThreads) {
            const float2 v = unpack2(tile[i]);
            y[t0 + i] = v;
        }
    }
    return true;
}

// One plain tile of a group's list (fir_plain_group_tiles).
struct PlainTileRef {
    const float2* x;
    const float* taps;
    float2* y;
    long long n;
    int num_taps;
    long long tile;
};

// The tiles i = 0 .. count - 1 of one group of 256 threads (source(i) gives tile i), two slots
// in flight: while tile i is computed from one slot, tile i + 1's samples arrive by bulk copy in
// the other, and tile i - 1's results leave by bulk store. Per tile the arithmetic, staging and
// results are fir_plain_tile's (same bits). Each slot (slot_bytes, at region + s * slot_bytes)
// holds an mbarrier at offset 0 and a tile in plain_layout(K) of its tile's K. `group_all`
// (a barrier of the group with an AND over its threads) also keeps the group in step. Returns
// false if a copy did not arrive within the wait limit (recorded in *fault; the group stops).
template <class Source, class Sync, class All>
__device__ __forceinline__ bool fir_plain_group_tiles(Source source, int count,
                                                      unsigned char* region, uint32_t slot_bytes,
                                                      unsigned int* fault, int tid, Sync sync,
                                                      All group_all)
{
    using namespace plain;
    if (count <= 0) {
        return true;
    }
    struct Geo {
        long long t0;
        long long base;
        int tile_len;
        bool interior;
        Layout lay;
    };
    auto geo = [](const PlainTileRef& r) {
        Geo g;
        g.lay = plain_layout(r.num_taps);
        g.t0 = r.tile * kTile;
        g.base = (g.t0 - (r.num_taps - 1)) & ~1ll;
        g.tile_len = static_cast<int>(g.t0 + kTile - g.base);
        g.interior = g.base >= 0 && g.t0 + kTile <= r.n;
        return g;
    };
    auto slot_of = [&](int s) { return region + static_cast<uint32_t>(s) * slot_bytes; };
    // Bulk copy of an interior tile's samples into slot s (tid 0).
    auto issue = [&](int s, const PlainTileRef& r, const Geo& g) {
        if (g.interior) {
            unsigned char* sl = slot_of(s);
            const uint32_t bar = smem_u32(sl);
            const uint32_t bytes = 8u * static_cast<uint32_t>(g.tile_len);
            fence_proxy_async_smem();   // after the slot's last generic reads
            mbar_arrive_expect_tx(bar, bytes);
            bulk_g2s(smem_u32(sl + g.lay.tile_off) + 8u * kGuard, r.x + g.base, bytes, bar);
        }
    };
    auto load_taps = [&](int s, const PlainTileRef& r, const Geo& g) {
        f32x2* taps2 = reinterpret_cast<f32x2*>(slot_of(s) + g.lay.taps_off);
        for (int k = tid; k < r.num_taps; k += kThreads) {
            const float h = __ldg(r.taps + k);
            taps2[k] = pack2(h, h);
        }
    };
    // The guard and, for tiles at either end of their capture, the samples (zero outside).
    auto fill = [&](int s, const PlainTileRef& r, const Geo& g) {
        f32x2* guard = reinterpret_cast<f32x2*>(slot_of(s) + g.lay.tile_off);
        f32x2* tile = guard + kGuard;
        if (tid < kGuard) {
            guard[tid] = 0ull;
        }
        if (!g.interior) {
            for (int i = tid; i < g.tile_len; i += kThreads) {
                const long long m = g.base + i;
                f32x2 v = 0ull;
                if (m >= 0 && m < r.n) {
                    const float2 q = r.x[m];
                    v = pack2(q.x, q.y);
                }
                tile[i] = v;
            }
        }
    };

    uint32_t phase[2] = {0u, 0u};
    if (tid == 0) {
        mbar_init(smem_u32(slot_of(0)), 1);
        mbar_init(smem_u32(slot_of(1)), 1);
        fence_mbar_init();
    }
    sync();
    PlainTileRef cur = source(0);
    {
        const Geo g = geo(cur);
        if (tid == 0) {
            issue(0, cur, g);
        }
        load_taps(0, cur, g);
        fill(0, cur, g);
    }
    sync();
    bool ok = true;
    for (int i = 0; i < count; ++i) {
        const int b = i & 1;
        const int nb = b ^ 1;
        const bool more = i + 1 < count;
        const PlainTileRef nxt = more ? source(i + 1) : cur;
        // Slot nb last held tile i - 1, whose results tid 0 stored from it.
        if (tid == 0) {
            bulk_wait_read_all();
            if (more) {
                issue(nb, nxt, geo(nxt));
            }
        }
        const Geo gc = geo(cur);
        unsigned char* sl = slot_of(b);
        f32x2* tile = reinterpret_cast<f32x2*>(sl + gc.lay.tile_off) + kGuard;
        if (gc.interior) {
            ok = mbar_wait_bounded(smem_u32(sl), phase[b], fault, kFaultTileLoad, nullptr);
            phase[b] ^= 1u;
        }
        const long long n0 = gc.t0 + static_cast<long long>(kR) * tid;
        f32x2 acc[kR];
        if (ok && n0 < cur.n) {
            compute_outputs(acc, tile, reinterpret_cast<f32x2*>(sl + gc.lay.taps_off),
                            static_cast<int>(n0 - gc.base), cur.num_taps);
        }
        sync();   // tile i read by every thread; tid 0's wait for slot nb done
        if (ok && n0 < cur.n) {
#pragma unroll
            for (int j = 0; j < kR; ++j) {
                tile[kR * tid + j] = acc[j];
            }
        }
        if (gc.interior) {
            fence_proxy_async_smem();
        }
        if (more) {
            // After the barrier above, so after tid 0 saw tile i - 1's store finish reading
            // slot nb: a longer filter's taps reach into where that tile's results were.
            load_taps(nb, nxt, geo(nxt));
            fill(nb, nxt, geo(nxt));
        }
        sync();
        if (gc.interior) {
            if (tid == 0 && ok) {
                bulk_s2g(cur.y + gc.t0, smem_u32(tile), 8u * kTile);
                bulk_commit();
            }
        } else if (ok) {
            const long long valid = cur.n - gc.t0 < kTile ? cur.n - gc.t0 : kTile;
            for (int k = tid; k < valid; k += kThreads) {
                cur.y[gc.t0 + k] = unpack2(tile[k]);
            }
        }
        // Every thread is past its reads of slot b before it is refilled (next iteration's
        // issue into slot (i + 2) & 1), and the group agrees on stopping.
        if (!group_all(ok)) {
            ok = false;
            break;
        }
        cur = nxt;
    }
    if (tid == 0) {
        bulk_wait_read_all();
    }
    return ok;
}

using plain::plain_layout;

}  // namespace rfx
