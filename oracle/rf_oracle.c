/*
 * rf_oracle.c — CPU restatement of the reference's complex-baseband filtering path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker, never the product: only tests/,
 * __graft_entry__.smoke() and bench.py (its cpu_baseline leg and its `--impl reference` arm)
 * may load it. The shipped library (gpu-rf-pipeline_gb300/) never links or calls it.
 *
 * What it restates (paths are inside the gpu-rf-pipeline project):
 *
 *   rfo_fir_f64             tools/reference.py:103-111   y[n] = sum_k h[k] x[n-k], x[m<0] = 0,
 *                                                         output length N, float64 arithmetic.
 *   rfo_fir_f32_seq         src/fir.cu:30-40             the reference GPU kernels' float32
 *                                                         arithmetic: one fused multiply-add per
 *                                                         tap, k ascending from 0, both I and Q,
 *                                                         accumulator starting at +0.0f. The
 *                                                         register kernel (src/fir.cu:377-395)
 *                                                         runs the same chain over a zero-padded
 *                                                         tile, which adds exact zeros only.
 *   rfo_channelize_f64      tools/reference.py:128-146   z[t][k] = sum_l h[l] x[tM-l] e^{+2pi i kl/M}
 *                                                         as M polyphase branch sums followed by
 *                                                         the unnormalized inverse DFT over m.
 *   rfo_channelize_branch_f32_seq
 *                           src/channelize.cu:25-49      the reference's branch-sum kernel in
 *                                                         float32: l = m, m+M, ... ascending,
 *                                                         one fused multiply-add per tap, stopping
 *                                                         at the start of the input.
 *
 * Build: see oracle/Makefile (compiled with -ffp-contract=off so that the only fused
 * multiply-adds are the explicit fmaf() calls of the float32 restatements).
 * Threads: every entry point takes a thread count and splits the OUTPUT range into contiguous
 * segments; each output is computed by one thread in a fixed order, so results do not depend on
 * the thread count.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RFO_PI 3.14159265358979323846264338327950288

typedef void (*rfo_range_fn)(void* ctx, int64_t begin, int64_t end);

struct rfo_job {
    rfo_range_fn fn;
    void* ctx;
    int64_t begin;
    int64_t end;
};

static void* rfo_thread_main(void* arg)
{
    struct rfo_job* job = (struct rfo_job*)arg;
    job->fn(job->ctx, job->begin, job->end);
    return NULL;
}

/* Runs fn over [0, count) split into `threads` contiguous pieces (the caller's thread does the
 * last piece). Falls back to a serial call when threads <= 1 or pthread_create fails. */
static void rfo_parallel(rfo_range_fn fn, void* ctx, int64_t count, int threads)
{
    if (threads > 256) {
        threads = 256;
    }
    if (threads <= 1 || count < 2 * (int64_t)threads) {
        fn(ctx, 0, count);
        return;
    }
    pthread_t tid[256];
    struct rfo_job jobs[256];
    int started[256];
    const int64_t step = (count + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = t * step < count ? t * step : count;
        jobs[t].end = (t + 1) * step < count ? (t + 1) * step : count;
        started[t] = 0;
    }
    for (int t = 0; t < threads - 1; ++t) {
        started[t] = pthread_create(&tid[t], NULL, rfo_thread_main, &jobs[t]) == 0;
        if (!started[t]) {
            fn(ctx, jobs[t].begin, jobs[t].end);
        }
    }
    fn(ctx, jobs[threads - 1].begin, jobs[threads - 1].end);
    for (int t = 0; t < threads - 1; ++t) {
        if (started[t]) {
            pthread_join(tid[t], NULL);
        }
    }
}

/* ---- FIR, float64 ------------------------------------------------------------------------ */

struct fir_ctx {
    const float* x;   /* interleaved I/Q, n samples */
    int64_t n;
    const float* h;
    int taps;
    double* y;        /* interleaved I/Q output */
    float* y32;       /* float32 output (sequential-FMA restatement) */
};

/* Block of outputs at a time so the inner loop over outputs vectorizes; every output still
 * sums its products in k order. */
#define RFO_FIR_BLOCK 64

static void fir_f64_range(void* vctx, int64_t begin, int64_t end)
{
    const struct fir_ctx* c = (const struct fir_ctx*)vctx;
    double acc_re[RFO_FIR_BLOCK];
    double acc_im[RFO_FIR_BLOCK];
    for (int64_t n0 = begin; n0 < end; n0 += RFO_FIR_BLOCK) {
        const int len = (int)((end - n0) < RFO_FIR_BLOCK ? (end - n0) : RFO_FIR_BLOCK);
        for (int j = 0; j < len; ++j) {
            acc_re[j] = 0.0;
            acc_im[j] = 0.0;
        }
        for (int k = 0; k < c->taps; ++k) {
            const double hk = (double)c->h[k];
            /* outputs n0 + j with n0 + j - k >= 0 */
            int j0 = (int)(k - n0);
            if (j0 < 0) {
                j0 = 0;
            }
            if (j0 >= len) {
                break; /* larger k only reaches further before the start of the input */
            }
            const float* xs = c->x + 2 * (n0 - k);
            for (int j = j0; j < len; ++j) {
                acc_re[j] += hk * (double)xs[2 * j];
                acc_im[j] += hk * (double)xs[2 * j + 1];
            }
        }
        for (int j = 0; j < len; ++j) {
            c->y[2 * (n0 + j)] = acc_re[j];
            c->y[2 * (n0 + j) + 1] = acc_im[j];
        }
    }
}

void rfo_fir_f64(const float* x_iq, int64_t n, const float* taps, int num_taps, double* y_iq,
                 int threads)
{
    struct fir_ctx c = {x_iq, n, taps, num_taps, y_iq, NULL};
    rfo_parallel(fir_f64_range, &c, n, threads);
}

/* ---- FIR, float32 in the reference kernels' order ---------------------------------------- */

static void fir_f32_range(void* vctx, int64_t begin, int64_t end)
{
    const struct fir_ctx* c = (const struct fir_ctx*)vctx;
    for (int64_t n = begin; n < end; ++n) {
        const int64_t last = n < (int64_t)c->taps - 1 ? n : (int64_t)c->taps - 1;
        float re = 0.0f;
        float im = 0.0f;
        for (int64_t k = 0; k <= last; ++k) {
            const float hk = c->h[k];
            re = fmaf(hk, c->x[2 * (n - k)], re);
            im = fmaf(hk, c->x[2 * (n - k) + 1], im);
        }
        c->y32[2 * n] = re;
        c->y32[2 * n + 1] = im;
    }
}

void rfo_fir_f32_seq(const float* x_iq, int64_t n, const float* taps, int num_taps,
                     float* y_iq, int threads)
{
    struct fir_ctx c = {x_iq, n, taps, num_taps, NULL, y_iq};
    rfo_parallel(fir_f32_range, &c, n, threads);
}

/* ---- channelizer ------------------------------------------------------------------------- */

int64_t rfo_channelize_frames(int64_t n, int channels)
{
    return channels > 0 ? (n + channels - 1) / channels : 0;
}

struct chan_ctx {
    const float* x;
    int64_t n;
    const float* h;
    int taps;
    int m;              /* channels */
    int log2m;          /* >= 0 when m is a power of two, else -1 */
    const double* tw;   /* tw[2j], tw[2j+1] = cos, sin(2 pi j / m), j < m */
    double* z;          /* frames * m interleaved I/Q, float64 */
    float* u32;         /* frames * m interleaved I/Q, float32 branch sums */
};

/* In-place unnormalized inverse DFT of one frame: out[k] = sum_m in[m] e^{+2 pi i k m / M}.
 * Power-of-two sizes use an iterative radix-2 decimation-in-time FFT (bit-reversed input order,
 * then log2(M) butterfly passes); other sizes use the direct sum with the twiddle table. */
static void inverse_dft(double* re, double* im, int m, int log2m, const double* tw,
                        double* scratch)
{
    if (m == 1) {
        return;
    }
    if (log2m < 0) {
        double* sre = scratch;
        double* sim = scratch + m;
        for (int k = 0; k < m; ++k) {
            double ar = 0.0;
            double ai = 0.0;
            int64_t idx = 0;
            for (int j = 0; j < m; ++j) {
                const double c = tw[2 * idx];
                const double s = tw[2 * idx + 1];
                ar += re[j] * c - im[j] * s;
                ai += re[j] * s + im[j] * c;
                idx += k;
                if (idx >= m) {
                    idx -= m;
                }
            }
            sre[k] = ar;
            sim[k] = ai;
        }
        memcpy(re, sre, sizeof(double) * (size_t)m);
        memcpy(im, sim, sizeof(double) * (size_t)m);
        return;
    }
    for (int i = 0; i < m; ++i) {
        int r = 0;
        for (int b = 0; b < log2m; ++b) {
            r |= ((i >> b) & 1) << (log2m - 1 - b);
        }
        if (r > i) {
            double t = re[i];
            re[i] = re[r];
            re[r] = t;
            t = im[i];
            im[i] = im[r];
            im[r] = t;
        }
    }
    for (int len = 2; len <= m; len <<= 1) {
        const int half = len >> 1;
        const int stride = m / len;
        for (int base = 0; base < m; base += len) {
            for (int j = 0; j < half; ++j) {
                const double c = tw[2 * (j * stride)];
                const double s = tw[2 * (j * stride) + 1];
                const int a = base + j;
                const int b = a + half;
                const double br = re[b] * c - im[b] * s;
                const double bi = re[b] * s + im[b] * c;
                re[b] = re[a] - br;
                im[b] = im[a] - bi;
                re[a] += br;
                im[a] += bi;
            }
        }
    }
}

static void chan_f64_range(void* vctx, int64_t begin, int64_t end)
{
    const struct chan_ctx* c = (const struct chan_ctx*)vctx;
    const int m = c->m;
    double* buf = (double*)malloc(sizeof(double) * 4 * (size_t)m);
    if (buf == NULL) {
        return;
    }
    double* re = buf;
    double* im = buf + m;
    double* scratch = buf + 2 * m;
    for (int64_t t = begin; t < end; ++t) {
        const int64_t newest = t * (int64_t)m; /* index of x[tM] */
        for (int b = 0; b < m; ++b) {
            double ar = 0.0;
            double ai = 0.0;
            for (int64_t l = b; l < c->taps; l += m) {
                const int64_t s = newest - l;
                if (s < 0) {
                    break;
                }
                if (s < c->n) {
                    ar += (double)c->h[l] * (double)c->x[2 * s];
                    ai += (double)c->h[l] * (double)c->x[2 * s + 1];
                }
            }
            re[b] = ar;
            im[b] = ai;
        }
        inverse_dft(re, im, m, c->log2m, c->tw, scratch);
        for (int k = 0; k < m; ++k) {
            c->z[2 * (newest + k)] = re[k];
            c->z[2 * (newest + k) + 1] = im[k];
        }
    }
    free(buf);
}

static int log2_exact(int m)
{
    int l = 0;
    while ((1 << l) < m) {
        ++l;
    }
    return (1 << l) == m ? l : -1;
}

int rfo_channelize_f64(const float* x_iq, int64_t n, const float* taps, int num_taps,
                       int channels, double* z_iq, int threads)
{
    if (channels < 1 || num_taps < 1) {
        return 1;
    }
    double* tw = (double*)malloc(sizeof(double) * 2 * (size_t)channels);
    if (tw == NULL) {
        return 2;
    }
    for (int j = 0; j < channels; ++j) {
        const double a = 2.0 * RFO_PI * (double)j / (double)channels;
        tw[2 * j] = cos(a);
        tw[2 * j + 1] = sin(a);
    }
    struct chan_ctx c = {x_iq, n, taps, num_taps, channels, log2_exact(channels), tw, z_iq,
                         NULL};
    rfo_parallel(chan_f64_range, &c, rfo_channelize_frames(n, channels), threads);
    free(tw);
    return 0;
}

static void chan_branch_f32_range(void* vctx, int64_t begin, int64_t end)
{
    const struct chan_ctx* c = (const struct chan_ctx*)vctx;
    const int m = c->m;
    for (int64_t idx = begin; idx < end; ++idx) {
        const int64_t t = idx / m;
        const int b = (int)(idx % m);
        const int64_t newest = t * (int64_t)m;
        float re = 0.0f;
        float im = 0.0f;
        for (int64_t l = b; l < c->taps; l += m) {
            const int64_t s = newest - l;
            if (s < 0) {
                break;
            }
            const float xr = s < c->n ? c->x[2 * s] : 0.0f;
            const float xi = s < c->n ? c->x[2 * s + 1] : 0.0f;
            re = fmaf(c->h[l], xr, re);
            im = fmaf(c->h[l], xi, im);
        }
        c->u32[2 * idx] = re;
        c->u32[2 * idx + 1] = im;
    }
}

int rfo_channelize_branch_f32_seq(const float* x_iq, int64_t n, const float* taps,
                                  int num_taps, int channels, float* u_iq, int threads)
{
    if (channels < 1 || num_taps < 1) {
        return 1;
    }
    struct chan_ctx c = {x_iq, n, taps, num_taps, channels, -1, NULL, NULL, u_iq};
    rfo_parallel(chan_branch_f32_range, &c, rfo_channelize_frames(n, channels) * channels,
                 threads);
    return 0;
}
