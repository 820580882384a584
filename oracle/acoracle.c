/*
 * CPU oracle for the Anime4KCPP CNN upscaling path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the arithmetic of the reference's CPU
 * processor so that the CUDA path of this repository can be checked against
 * it.  Only tests, the smoke check and the CPU-baseline leg of the benchmark
 * use it; the product library never links or calls it.
 *
 * Two families of functions:
 *   - "ref order" FP32 functions reproduce the reference's Generic backend
 *     operation by operation (same products, same left-to-right sums, no
 *     fused multiply-add; build with -ffp-contract=off), so they are
 *     bit-identical to the reference's own Generic CPU processor;
 *   - FP64 functions run the same network in double precision and return
 *     unquantised outputs, used for the max-abs-error / PSNR statistics.
 *
 * Reference files followed (paths inside the Anime4KCPP project):
 *   core/internal/AC/Core/Internal/Util.hpp:50-78            toFloat / fromFloat
 *   core/internal/AC/Core/Internal/Processor/CPU/Common.hpp   layer templates
 *       :116-164 conv3x3_float, :166-197 conv3x3_cin1, :223-288 conv3x3_conv1x1,
 *       :290-342 conv3x3_pixelshuffle, :344-393 conv3x3_deconv2x2
 *   core/internal/AC/Core/Internal/Processor/CPU/Generic.hpp:19-81  summation order
 *   core/src/processor/cpu/CPUProcessor.cpp:1371-1390 (ACNetLegacy), :1417-1436 (ACNet<8>),
 *       :1464-1491 (ARNet), :1519-1600 (ArtCNN<16/32>), :1629-1715 (FSRCNNX<8/16>)
 *   core/src/ImageProcess.cpp:39-61 rgb2yuv, :114-138 rgba2yuva,
 *       :192-215 yuv2rgb, :276-308 yuva2rgba
 *   core/src/ImageResize.cpp:62-83,127-134,136-273  resize filters (the
 *       sampling itself is done by stb_image_resize2 in the reference, which is
 *       not vendored; orc_resize below is this project's own restatement)
 *
 * Parity status: the FP32 luma network and colour conversion are pinned
 * against the reference's own CPU code compiled from its sources (golden
 * vectors under tests/golden/); the chroma resize is a restatement of the
 * filter definition and is not pinned to stb_image_resize2.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_U8 0x001
#define ORC_U16 0x002
#define ORC_F32 0x204

/* ---------------------------------------------------------------- helpers */

/* Util.hpp:50-61 toFloat: unsigned -> v / max, float as is. */
static inline float to_float(const void* base, size_t idx, int type)
{
    switch (type)
    {
    case ORC_U8: return (float)((const uint8_t*)base)[idx] / 255.0f;
    case ORC_U16: return (float)((const uint16_t*)base)[idx] / 65535.0f;
    default: return ((const float*)base)[idx];
    }
}
static inline double to_double(const void* base, size_t idx, int type)
{
    switch (type)
    {
    case ORC_U8: return (double)((const uint8_t*)base)[idx] / 255.0;
    case ORC_U16: return (double)((const uint16_t*)base)[idx] / 65535.0;
    default: return (double)((const float*)base)[idx];
    }
}
/* Util.hpp:63-78 fromFloat: saturate to [0,1], then v*max + 0.5 truncated. */
static inline void from_float(void* base, size_t idx, int type, float v)
{
    float s = v < 0.0f ? 0.0f : (v < 1.0f ? v : 1.0f);
    switch (type)
    {
    case ORC_U8: { float t = s * 255.0f; t = t + 0.5f; ((uint8_t*)base)[idx] = (uint8_t)t; break; }
    case ORC_U16: { float t = s * 65535.0f; t = t + 0.5f; ((uint16_t*)base)[idx] = (uint16_t)t; break; }
    default: ((float*)base)[idx] = s; break;
    }
}

static inline const void* rowp(const void* base, int stride, int y) { return (const uint8_t*)base + (size_t)stride * y; }
static inline void* rowpw(void* base, int stride, int y) { return (uint8_t*)base + (size_t)stride * y; }

/* std::max(v, 0.0f) returns v unless v < 0 (keeps -0.0f); mirror that exactly. */
static inline float std_max0(float v) { return (v < 0.0f) ? 0.0f : v; }
static inline float std_min0(float v) { return (0.0f < v) ? 0.0f : v; }

/* ------------------------------------------------------------ row threads */

typedef void (*row_fn)(void* ctx, int y0, int y1);
typedef struct { row_fn fn; void* ctx; int y0, y1; } row_job;
static void* row_thread(void* p)
{
    row_job* j = (row_job*)p;
    j->fn(j->ctx, j->y0, j->y1);
    return NULL;
}
static void parallel_rows(row_fn fn, void* ctx, int h, int threads)
{
    if (threads <= 1 || h < 2)
    {
        fn(ctx, 0, h);
        return;
    }
    if (threads > h) threads = h;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    row_job jobs[256];
    int started = 0;
    for (int t = 0; t < threads; t++)
    {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].y0 = (int)((long long)h * t / threads);
        jobs[t].y1 = (int)((long long)h * (t + 1) / threads);
        if (t == threads - 1) break;
        if (pthread_create(&tid[t], NULL, row_thread, &jobs[t]) == 0) started++;
        else { fn(ctx, jobs[t].y0, jobs[t].y1); tid[t] = 0; }
    }
    fn(ctx, jobs[threads - 1].y0, jobs[threads - 1].y1);
    for (int t = 0; t < threads - 1; t++)
        if (tid[t]) pthread_join(tid[t], NULL);
    (void)started;
}

/* ----------------------------------------------- FP32 layers (ref order) */

enum { ACT_IDENTITY = 0, ACT_RELU = 1, ACT_PRELU = 2 };

static inline float activate(float v, int act, const float* alphas, int n)
{
    if (act == ACT_RELU) return std_max0(v);
    if (act == ACT_PRELU)
    {
        float a = std_max0(v);
        float b = alphas[n] * std_min0(v);
        return a + b;
    }
    return v;
}

/* Gather the 3x3 clamped neighbourhood of (x, y): Common.hpp:121-143. */
static inline void taps3x3(int x, int y, int w, int h, int* xs, int* ys)
{
    int lp = x > 0 ? 1 : 0, rp = x < w - 1 ? 1 : 0;
    int tp = y > 0 ? 1 : 0, bp = y < h - 1 ? 1 : 0;
    xs[0] = x - lp; xs[1] = x; xs[2] = x + rp;
    ys[0] = y - tp; ys[1] = y; ys[2] = y + bp;
}

/* Layer 0: conv3x3 1->8 (+bias, activation).  Generic.hpp:62-69:
 * out[n] = ((((p0 + p1) + p2) ... + p8) + bias[n]. */
typedef struct {
    const void* src; int w, h, sstride, type;
    float* dst; /* h*w*8 */
    const float* k; const float* b; int act; const float* alphas;
} l0_ctx;
static void l0_rows(void* p, int y0, int y1)
{
    l0_ctx* c = (l0_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            float r[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    r[i * 3 + j] = to_float(rowp(c->src, c->sstride, ys[i]), (size_t)xs[j], c->type);
            float* out = c->dst + ((size_t)y * c->w + x) * 8;
            for (int n = 0; n < 8; n++)
            {
                const float* kp = c->k + n * 9;
                float s = r[0] * kp[0];
                for (int t = 1; t < 9; t++) { float m = r[t] * kp[t]; s = s + m; }
                s = s + c->b[n];
                out[n] = activate(s, c->act, c->alphas, n);
            }
        }
}

/* 3x3 conv cin=8 -> cout (8 or 4) accumulation, Generic.hpp:71-80:
 * for c: sum += (((r0[c]k0[c] + r1[c]k1[c]) + ...) + r8[c]k8[c]); out = sum + bias. */
static inline void conv8_sum(const float* const* rp, const float* k, const float* b, int cout, float* out)
{
    for (int n = 0; n < cout; n++)
    {
        const float* kn = k + n * 72;
        float sum = 0.0f;
        for (int c = 0; c < 8; c++)
        {
            float blk = rp[0][c] * kn[c];
            for (int p = 1; p < 9; p++) { float m = rp[p][c] * kn[p * 8 + c]; blk = blk + m; }
            sum = sum + blk;
        }
        out[n] = sum + b[n];
    }
}

/* conv3x3 8->8 with activation and optional residual "sum*scale + id". */
typedef struct {
    const float* src; float* dst; int w, h;
    const float* k; const float* b; int act; const float* alphas;
    const float* id; float scale;
} l8_ctx;
static void l8_rows(void* p, int y0, int y1)
{
    l8_ctx* c = (l8_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * 8;
            float sum[8];
            conv8_sum(rp, c->k, c->b, 8, sum);
            float* out = c->dst + ((size_t)y * c->w + x) * 8;
            const float* idp = c->id ? c->id + ((size_t)y * c->w + x) * 8 : NULL;
            for (int n = 0; n < 8; n++)
            {
                float v = activate(sum[n], c->act, c->alphas, n);
                if (idp) { float m = v * c->scale; v = m + idp[n]; }
                out[n] = v;
            }
        }
}

/* Last ACNetLegacy layer: conv3x3 8->8 + ReLU, then deconv 2x2 stride 2 8->1
 * (Common.hpp:344-393): out(2x+dx, 2y+dy) = fromFloat(dot8(s, k2 + 8*(2dy+dx))). */
typedef struct {
    const float* src; int w, h;
    void* dst; int dstride, type;
    const float* k; const float* b; const float* k2;
} ld_ctx;
static void ld_rows(void* p, int y0, int y1)
{
    ld_ctx* c = (ld_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * 8;
            float s[8];
            conv8_sum(rp, c->k, c->b, 8, s);
            for (int n = 0; n < 8; n++) s[n] = std_max0(s[n]);
            for (int dy = 0; dy < 2; dy++)
            {
                void* row = rowpw(c->dst, c->dstride, 2 * y + dy);
                for (int dx = 0; dx < 2; dx++)
                {
                    const float* k2 = c->k2 + 8 * (dy * 2 + dx);
                    float d = s[0] * k2[0];
                    for (int i = 1; i < 8; i++) { float m = s[i] * k2[i]; d = d + m; }
                    from_float(row, (size_t)(2 * x + dx), c->type, d);
                }
            }
        }
}

/* ARNet tail part 1: conv3x3 8->8 identity + residual (scale, id), then
 * conv1x1 8->8 + PReLU + feat (Common.hpp:223-288). */
typedef struct {
    const float* src; float* dst; int w, h;
    const float* k1; const float* b1; const float* id; float scale;
    const float* k2; const float* b2; const float* a2; const float* feat;
} lt_ctx;
static void lt_rows(void* p, int y0, int y1)
{
    lt_ctx* c = (lt_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * 8;
            size_t off = ((size_t)y * c->w + x) * 8;
            float buf[8];
            conv8_sum(rp, c->k1, c->b1, 8, buf);
            for (int n = 0; n < 8; n++) { float m = buf[n] * c->scale; buf[n] = m + c->id[off + n]; }
            for (int n = 0; n < 8; n++)
            {
                const float* kn = c->k2 + n * 8;
                float sum = 0.0f;
                for (int i = 0; i < 8; i++) { float m = buf[i] * kn[i]; sum = sum + m; }
                sum = sum + c->b2[n];
                float v = activate(sum, ACT_PRELU, c->a2, n);
                float m = v * 1.0f;
                c->dst[off + n] = m + c->feat[off + n];
            }
        }
}

/* ARNet upscale: conv3x3 8->4 identity, pixel-shuffle, + nearest toFloat(src)
 * (Common.hpp:290-342). */
typedef struct {
    const float* src; int w, h;
    const void* lum; int lstride;
    void* dst; int dstride, type;
    const float* k; const float* b;
} lp_ctx;
static void lp_rows(void* p, int y0, int y1)
{
    lp_ctx* c = (lp_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * 8;
            float s[4];
            conv8_sum(rp, c->k, c->b, 4, s);
            float near = to_float(rowp(c->lum, c->lstride, y), (size_t)x, c->type);
            for (int n = 0; n < 4; n++)
            {
                float m = s[n] * 1.0f;
                float v = m + near;
                from_float(rowpw(c->dst, c->dstride, 2 * y + (n >> 1)), (size_t)(2 * x + (n & 1)), c->type, v);
            }
        }
}

/* --------------------------------------------------------- public FP32 API */

/* ACNetLegacy x2 pass, CPUProcessor.cpp:1371-1390.  kernels: 4712 floats,
 * biases: 72 floats in the reference's NHWC layout (ACNet.hpp:34-60). */
int orc_acnet_legacy_x2(const void* src, int w, int h, int sstride, int type,
                        void* dst, int dstride, const float* kernels, const float* biases, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0) return -22;
    size_t n = (size_t)w * h * 8;
    float* a = (float*)malloc(n * sizeof(float));
    float* b = (float*)malloc(n * sizeof(float));
    if (!a || !b) { free(a); free(b); return -12; }
    l0_ctx c0 = { src, w, h, sstride, type, a, kernels, biases, ACT_RELU, NULL };
    parallel_rows(l0_rows, &c0, h, threads);
    for (int l = 1; l < 8; l++)
    {
        l8_ctx c = { a, b, w, h, kernels + 72 + 576 * (l - 1), biases + 8 * l, ACT_RELU, NULL, NULL, 0.0f };
        parallel_rows(l8_rows, &c, h, threads);
        float* t = a; a = b; b = t;
    }
    ld_ctx cd = { a, w, h, dst, dstride, type, kernels + 72 + 576 * 7, biases + 64, kernels + 72 + 576 * 8 };
    parallel_rows(ld_rows, &cd, h, threads);
    free(a);
    free(b);
    return 0;
}

/* ------------------------- 4-lane form of the reference's NEON backend */

/* ACNetLegacy x2 in the operation order of the reference's NEON backend
 * (core/internal/AC/Core/Internal/Processor/CPU/ARM/NEON.hpp, the backend
 * its CPU processor selects on aarch64), written with portable 4-lane
 * vectors (GCC vector extensions: NEON on aarch64, SSE on x86_64):
 *
 *   conv_cin1 (layer 0, 9 taps): s = r[0..3]*k[0..3] + r[4..7]*k[4..7] in 4
 *     lanes, sum = hsum(s) + r[8]*k[8], out = sum + bias;
 *   conv 8 -> 8 (conv_kernel with 4-lane groups): s[n] accumulates
 *     r_p[4i..4i+3] * k[n][p][4i..4i+3] over taps p = 0..8 and i = 0, 1;
 *     out[n] = bias[n] + hsum(s[n]);
 *   dot<8> (the 2x2 transposed conv): hsum(s[0..3]*k[0..3] + s[4..7]*k[4..7]);
 *   hsum(v) = (v0 + v1) + (v2 + v3) (pairwise adds).
 *
 * Multiply and add are separate roundings (vmlaq_f32's definition; this
 * file is compiled without contraction).  Used as the timed CPU baseline of
 * the reference's path on the GPU host; pinned to the reference's Generic
 * output within its own ISA spread (1 LSB). */
typedef float v4f __attribute__((vector_size(16)));

static inline v4f v4_load(const float* p)
{
    v4f v;
    memcpy(&v, p, sizeof(v));
    return v;
}
static inline float v4_hsum(v4f v) { return (v[0] + v[1]) + (v[2] + v[3]); }

typedef struct {
    const void* src; int w, h, sstride, type;
    const float* in; float* out;
    void* dst; int dstride;
    const float* k; const float* b; const float* k2;
} s4_ctx;

static void s4_l0_rows(void* p, int y0, int y1)
{
    s4_ctx* c = (s4_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            float r[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    r[i * 3 + j] = to_float(rowp(c->src, c->sstride, ys[i]), (size_t)xs[j], c->type);
            const v4f r0 = v4_load(r), r1 = v4_load(r + 4);
            float* out = c->out + ((size_t)y * c->w + x) * 8;
            for (int n = 0; n < 8; n++)
            {
                const float* kp = c->k + n * 9;
                v4f acc = r0 * v4_load(kp);
                acc = acc + r1 * v4_load(kp + 4);
                float sum = v4_hsum(acc);
                float m = r[8] * kp[8];
                sum = sum + m;
                out[n] = std_max0(sum + c->b[n]);
            }
        }
}

static inline void s4_conv8(const float* const* rp, const float* k, const float* b, float* out)
{
    v4f acc[8];
    for (int n = 0; n < 8; n++) acc[n] = (v4f){0.0f, 0.0f, 0.0f, 0.0f};
    for (int t = 0; t < 9; t++)
        for (int i = 0; i < 2; i++)
        {
            const v4f r = v4_load(rp[t] + 4 * i);
            for (int n = 0; n < 8; n++) acc[n] = acc[n] + r * v4_load(k + n * 72 + t * 8 + 4 * i);
        }
    for (int n = 0; n < 8; n++) out[n] = b[n] + v4_hsum(acc[n]);
}

static void s4_l8_rows(void* p, int y0, int y1)
{
    s4_ctx* c = (s4_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->in + ((size_t)ys[i] * c->w + xs[j]) * 8;
            float* out = c->out + ((size_t)y * c->w + x) * 8;
            s4_conv8(rp, c->k, c->b, out);
            for (int n = 0; n < 8; n++) out[n] = std_max0(out[n]);
        }
}

static void s4_last_rows(void* p, int y0, int y1)
{
    s4_ctx* c = (s4_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->in + ((size_t)ys[i] * c->w + xs[j]) * 8;
            float s[8];
            s4_conv8(rp, c->k, c->b, s);
            for (int n = 0; n < 8; n++) s[n] = std_max0(s[n]);
            const v4f s0 = v4_load(s), s1 = v4_load(s + 4);
            for (int dy = 0; dy < 2; dy++)
            {
                void* row = rowpw(c->dst, c->dstride, 2 * y + dy);
                for (int dx = 0; dx < 2; dx++)
                {
                    const float* k2 = c->k2 + 8 * (dy * 2 + dx);
                    v4f acc = s0 * v4_load(k2);
                    acc = acc + s1 * v4_load(k2 + 4);
                    from_float(row, (size_t)(2 * x + dx), c->type, v4_hsum(acc));
                }
            }
        }
}

int orc_acnet_legacy_x2_simd4(const void* src, int w, int h, int sstride, int type,
                              void* dst, int dstride, const float* kernels, const float* biases, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0) return -22;
    size_t n = (size_t)w * h * 8;
    float* a = (float*)malloc(n * sizeof(float));
    float* b = (float*)malloc(n * sizeof(float));
    if (!a || !b) { free(a); free(b); return -12; }
    s4_ctx c;
    memset(&c, 0, sizeof(c));
    c.src = src; c.w = w; c.h = h; c.sstride = sstride; c.type = type; c.dst = dst; c.dstride = dstride;
    c.out = a; c.k = kernels; c.b = biases;
    parallel_rows(s4_l0_rows, &c, h, threads);
    for (int l = 1; l < 8; l++)
    {
        c.in = a; c.out = b; c.k = kernels + 72 + 576 * (l - 1); c.b = biases + 8 * l;
        parallel_rows(s4_l8_rows, &c, h, threads);
        float* t = a; a = b; b = t;
    }
    c.in = a; c.k = kernels + 72 + 576 * 7; c.b = biases + 64; c.k2 = kernels + 72 + 576 * 8;
    parallel_rows(s4_last_rows, &c, h, threads);
    free(a);
    free(b);
    return 0;
}

/* ARNet<8> x2 pass, CPUProcessor.cpp:1464-1491; weight offsets ARNet.hpp:26-70. */
int orc_arnet_x2(const void* src, int w, int h, int sstride, int type,
                 void* dst, int dstride, const float* kernels, const float* biases, const float* alphas,
                 int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 2) return -22;
    size_t n = (size_t)w * h * 8;
    float* feat = (float*)malloc(n * sizeof(float));
    float* t1 = (float*)malloc(n * sizeof(float));
    float* t2 = (float*)malloc(n * sizeof(float));
    float* t3 = (float*)malloc(n * sizeof(float));
    if (!feat || !t1 || !t2 || !t3) { free(feat); free(t1); free(t2); free(t3); return -12; }
#define KOFF(l) ((l) <= 0 ? 0 : 72 + 576 * ((l) - 1))
#define AOFF(l) (8 * (((l) - 1) / 2))
    int l = 0;
    l0_ctx c0 = { src, w, h, sstride, type, feat, kernels, biases, ACT_IDENTITY, NULL };
    parallel_rows(l0_rows, &c0, h, threads); l++;
    {
        l8_ctx c = { feat, t1, w, h, kernels + KOFF(l), biases + 8 * l, ACT_PRELU, alphas + AOFF(l), NULL, 0.0f };
        parallel_rows(l8_rows, &c, h, threads); l++;
    }
    {
        l8_ctx c = { t1, t2, w, h, kernels + KOFF(l), biases + 8 * l, ACT_IDENTITY, NULL, feat, 0.2f };
        parallel_rows(l8_rows, &c, h, threads); l++;
    }
    for (int i = 0; i < blocks - 2; i++)
    {
        l8_ctx ca = { t2, t1, w, h, kernels + KOFF(l), biases + 8 * l, ACT_PRELU, alphas + AOFF(l), NULL, 0.0f };
        parallel_rows(l8_rows, &ca, h, threads); l++;
        l8_ctx cb = { t1, t3, w, h, kernels + KOFF(l), biases + 8 * l, ACT_IDENTITY, NULL, t2, 0.2f };
        parallel_rows(l8_rows, &cb, h, threads); l++;
        float* t = t2; t2 = t3; t3 = t;
    }
    {
        l8_ctx c = { t2, t1, w, h, kernels + KOFF(l), biases + 8 * l, ACT_PRELU, alphas + AOFF(l), NULL, 0.0f };
        parallel_rows(l8_rows, &c, h, threads); l++;
    }
    {
        /* layer l: 3x3 identity residual; layer l+1: 1x1 + PReLU (alpha index blocks) + feat */
        lt_ctx c = { t1, t3, w, h, kernels + KOFF(l), biases + 8 * l, t2, 0.2f,
                     kernels + 72 + 576 * (2 * blocks), biases + 8 * (l + 1), alphas + 8 * blocks, feat };
        parallel_rows(lt_rows, &c, h, threads); l += 2;
    }
    {
        lp_ctx c = { t3, w, h, src, sstride, dst, dstride, type,
                     kernels + 72 + 576 * (2 * blocks) + 64, biases + 8 * l };
        parallel_rows(lp_rows, &c, h, threads);
    }
#undef KOFF
#undef AOFF
    free(feat); free(t1); free(t2); free(t3);
    return 0;
}

/* ACNet<8> x2 pass, CPUProcessor.cpp:1417-1436: conv3x3_1to8_prelu, `blocks` x
 * conv3x3_8to8_prelu, conv3x3_8to4_identity_pixelshuffle_4to1_add.  Weight
 * offsets ACNet.hpp:93-114: layer l's kernels at 72 + 576 (l - 1), biases and
 * PReLU slopes at 8 l. */
int orc_acnet8_x2(const void* src, int w, int h, int sstride, int type,
                  void* dst, int dstride, const float* kernels, const float* biases, const float* alphas,
                  int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 1) return -22;
    size_t n = (size_t)w * h * 8;
    float* a = (float*)malloc(n * sizeof(float));
    float* b = (float*)malloc(n * sizeof(float));
    if (!a || !b) { free(a); free(b); return -12; }
    l0_ctx c0 = { src, w, h, sstride, type, a, kernels, biases, ACT_PRELU, alphas };
    parallel_rows(l0_rows, &c0, h, threads);
    for (int l = 1; l <= blocks; l++)
    {
        l8_ctx c = { a, b, w, h, kernels + 72 + 576 * (l - 1), biases + 8 * l, ACT_PRELU, alphas + 8 * l, NULL, 0.0f };
        parallel_rows(l8_rows, &c, h, threads);
        float* t = a; a = b; b = t;
    }
    lp_ctx cp = { a, w, h, src, sstride, dst, dstride, type, kernels + 72 + 576 * blocks, biases + 8 * (blocks + 1) };
    parallel_rows(lp_rows, &cp, h, threads);
    free(a);
    free(b);
    return 0;
}

/* ---------------------------- generic-width layers (ArtCNN, FSRCNNX) */

/* conv KxK (K = 3 or 5) 1 -> cout from the input plane, taps clamped to the
 * plane (Common.hpp:166-197 conv3x3_cin1, :196-222 conv5x5_cin1), Generic
 * conv_cin1 order (Generic.hpp:59-66: left-folded dot, then + bias), then
 * the activation. */
typedef struct {
    const void* src; int w, h, sstride, type;
    float* dst; int cout, K;
    const float* k; const float* b; int act; const float* alphas;
} g0_ctx;
static void g0_rows(void* p, int y0, int y1)
{
    g0_ctx* c = (g0_ctx*)p;
    const int K = c->K, R = K / 2;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            float r[25];
            for (int i = 0; i < K; i++)
            {
                int yy = y + i - R;
                yy = yy < 0 ? 0 : (yy > c->h - 1 ? c->h - 1 : yy);
                for (int j = 0; j < K; j++)
                {
                    int xx = x + j - R;
                    xx = xx < 0 ? 0 : (xx > c->w - 1 ? c->w - 1 : xx);
                    r[i * K + j] = to_float(rowp(c->src, c->sstride, yy), (size_t)xx, c->type);
                }
            }
            float* out = c->dst + ((size_t)y * c->w + x) * c->cout;
            for (int n = 0; n < c->cout; n++)
            {
                const float* kp = c->k + n * K * K;
                float s = r[0] * kp[0];
                for (int t = 1; t < K * K; t++) { float m = r[t] * kp[t]; s = s + m; }
                s = s + c->b[n];
                out[n] = activate(s, c->act, c->alphas, n);
            }
        }
}

/* Generic conv<cin, cout, 9> (Generic.hpp:70-80): per output channel n, sum
 * from 0 over input channels c of the left-folded tap products
 * rp[p][c] * k[n*cin*9 + p*cin + c], then + bias. */
static inline void convg_sum(const float* const* rp, const float* k, const float* b, int cin, int cout, float* out)
{
    for (int n = 0; n < cout; n++)
    {
        const float* kn = k + n * cin * 9;
        float sum = 0.0f;
        for (int c = 0; c < cin; c++)
        {
            float blk = rp[0][c] * kn[c];
            for (int p = 1; p < 9; p++) { float m = rp[p][c] * kn[p * cin + c]; blk = blk + m; }
            sum = sum + blk;
        }
        out[n] = sum + b[n];
    }
}

/* conv3x3 cin -> cout + activation, optional residual sum*scale + id
 * (Common.hpp:116-164). */
typedef struct {
    const float* src; float* dst; int w, h, cin, cout;
    const float* k; const float* b; int act; const float* alphas;
    const float* id; float scale;
} gc_ctx;
static void gc_rows(void* p, int y0, int y1)
{
    gc_ctx* c = (gc_ctx*)p;
    float sum[32];
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * c->cin;
            convg_sum(rp, c->k, c->b, c->cin, c->cout, sum);
            size_t off = ((size_t)y * c->w + x) * c->cout;
            for (int n = 0; n < c->cout; n++)
            {
                float v = activate(sum[n], c->act, c->alphas, n);
                if (c->id) { float m = v * c->scale; v = m + c->id[off + n]; }
                c->dst[off + n] = v;
            }
        }
}

/* FSRCNNX tail (Common.hpp:223-288 with postactive1x1): conv3x3 F -> F +
 * PReLU(a1), conv1x1 F -> F + bias, + feat, then PReLU(a2). */
typedef struct {
    const float* src; float* dst; int w, h, F;
    const float* k1; const float* b1; const float* a1;
    const float* k2; const float* b2; const float* a2; const float* feat;
} gt_ctx;
static void gt_rows(void* p, int y0, int y1)
{
    gt_ctx* c = (gt_ctx*)p;
    const int F = c->F;
    float buf[32];
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * F;
            convg_sum(rp, c->k1, c->b1, F, F, buf);
            for (int n = 0; n < F; n++) buf[n] = activate(buf[n], ACT_PRELU, c->a1, n);
            size_t off = ((size_t)y * c->w + x) * F;
            for (int n = 0; n < F; n++)
            {
                const float* kn = c->k2 + n * F;
                float sum = 0.0f;
                for (int i = 0; i < F; i++) { float m = buf[i] * kn[i]; sum = sum + m; }
                sum = sum + c->b2[n];
                float m = sum * 1.0f;
                sum = m + c->feat[off + n];
                c->dst[off + n] = activate(sum, ACT_PRELU, c->a2, n);
            }
        }
}

/* conv3x3 F -> 4, identity, pixel shuffle 2x2, fromFloat; no nearest add
 * (Common.hpp:290-342 without the interpolation argument). */
typedef struct {
    const float* src; int w, h, F;
    void* dst; int dstride, type;
    const float* k; const float* b;
} gp_ctx;
static void gp_rows(void* p, int y0, int y1)
{
    gp_ctx* c = (gp_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            const float* rp[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    rp[i * 3 + j] = c->src + ((size_t)ys[i] * c->w + xs[j]) * c->F;
            float s[4];
            convg_sum(rp, c->k, c->b, c->F, 4, s);
            for (int n = 0; n < 4; n++)
                from_float(rowpw(c->dst, c->dstride, 2 * y + (n >> 1)), (size_t)(2 * x + (n & 1)), c->type, s[n]);
        }
}

/* ArtCNN<F> x2 pass, CPUProcessor.cpp:1519-1545 / :1574-1600 (F = 16 / 32): head conv3x3
 * 1->F identity -> feat; conv F->F + ReLU, blocks-1 more; conv F->F identity
 * + feat; conv F->4 + pixel shuffle.  Offsets ArtCNN.hpp:44-56. */
int orc_artcnn_x2(const void* src, int w, int h, int sstride, int type,
                  void* dst, int dstride, const float* kernels, const float* biases, int F, int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 1 || F < 1 || F > 32) return -22;
    size_t n = (size_t)w * h * F;
    float* feat = (float*)malloc(n * sizeof(float));
    float* a = (float*)malloc(n * sizeof(float));
    float* b = (float*)malloc(n * sizeof(float));
    if (!feat || !a || !b) { free(feat); free(a); free(b); return -12; }
    g0_ctx c0 = { src, w, h, sstride, type, feat, F, 3, kernels, biases, ACT_IDENTITY, NULL };
    parallel_rows(g0_rows, &c0, h, threads);
    const float* in = feat;
    int l = 1;
    for (int i = 0; i < blocks; i++, l++)
    {
        gc_ctx c = { in, a, w, h, F, F, kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l, ACT_RELU, NULL, NULL, 0.0f };
        parallel_rows(gc_rows, &c, h, threads);
        in = a; float* t = a; a = b; b = t;
    }
    {
        gc_ctx c = { in, a, w, h, F, F, kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l, ACT_IDENTITY, NULL, feat, 1.0f };
        parallel_rows(gc_rows, &c, h, threads);
        in = a; l++;
    }
    gp_ctx cp = { in, w, h, F, dst, dstride, type, kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l };
    parallel_rows(gp_rows, &cp, h, threads);
    free(feat); free(a); free(b);
    return 0;
}

/* FSRCNNX<F> x2 pass, CPUProcessor.cpp:1629-1657 / :1687-1715 (F = 8 / 16): head conv5x5
 * 1->F identity -> feat; conv F->F + PReLU, blocks-2 more; conv F->F + PReLU
 * fused with conv1x1 F->F + feat + PReLU; conv F->4 + pixel shuffle.
 * Offsets FSRCNNX.hpp:46-66 (slopes of layer l at F (l-1)). */
int orc_fsrcnnx_x2(const void* src, int w, int h, int sstride, int type,
                   void* dst, int dstride, const float* kernels, const float* biases, const float* alphas,
                   int F, int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 2 || F < 1 || F > 32) return -22;
    size_t n = (size_t)w * h * F;
    float* feat = (float*)malloc(n * sizeof(float));
    float* a = (float*)malloc(n * sizeof(float));
    float* b = (float*)malloc(n * sizeof(float));
    if (!feat || !a || !b) { free(feat); free(a); free(b); return -12; }
    g0_ctx c0 = { src, w, h, sstride, type, feat, F, 5, kernels, biases, ACT_IDENTITY, NULL };
    parallel_rows(g0_rows, &c0, h, threads);
    const float* in = feat;
    int l = 1;
    for (; l < blocks; l++)
    {
        gc_ctx c = { in, a, w, h, F, F, kernels + F * 25 + F * F * 9 * (l - 1), biases + F * l, ACT_PRELU,
                     alphas + F * (l - 1), NULL, 0.0f };
        parallel_rows(gc_rows, &c, h, threads);
        in = a; float* t = a; a = b; b = t;
    }
    {
        gt_ctx c = { in, a, w, h, F, kernels + F * 25 + F * F * 9 * (l - 1), biases + F * l, alphas + F * (l - 1),
                     kernels + F * 25 + F * F * 9 * blocks, biases + F * (l + 1), alphas + F * l, feat };
        parallel_rows(gt_rows, &c, h, threads);
        in = a; l += 2;
    }
    gp_ctx cp = { in, w, h, F, dst, dstride, type, kernels + F * 25 + F * F * 9 * blocks + F * F, biases + F * l };
    parallel_rows(gp_rows, &cp, h, threads);
    free(feat); free(a); free(b);
    return 0;
}

/* ------------------------------------------------------- FP64 networks */

static inline void taps_d(const double* src, int w, int x, int y, int h, const double** rp)
{
    int xs[3], ys[3];
    taps3x3(x, y, w, h, xs, ys);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            rp[i * 3 + j] = src + ((size_t)ys[i] * w + xs[j]) * 8;
}
static inline void conv8_d(const double* const* rp, const float* k, const float* b, int cout, double* out)
{
    for (int n = 0; n < cout; n++)
    {
        double s = 0.0;
        for (int p = 0; p < 9; p++)
            for (int c = 0; c < 8; c++) s += rp[p][c] * (double)k[n * 72 + p * 8 + c];
        out[n] = s + (double)b[n];
    }
}
static inline double act_d(double v, int act, const float* alphas, int n)
{
    if (act == ACT_RELU) return v > 0.0 ? v : 0.0;
    if (act == ACT_PRELU) return v > 0.0 ? v : (double)alphas[n] * v;
    return v;
}

typedef struct {
    const void* src; int w, h, sstride, type;
    double* a; double* b; double* feat; double* t3;
    double* dst; /* (2h) x (2w) unquantised */
    const float* k; const float* bi; const float* al; int blocks;
    int stage; /* which layer to run */
    const double* in; double* out; int act; const float* alpha_l; const double* id; double scale;
    const float* kl; const float* bl;
} d_ctx;

static void d_l0_rows(void* p, int y0, int y1)
{
    d_ctx* c = (d_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            int xs[3], ys[3];
            taps3x3(x, y, c->w, c->h, xs, ys);
            double r[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    r[i * 3 + j] = to_double(rowp(c->src, c->sstride, ys[i]), (size_t)xs[j], c->type);
            double* o = c->out + ((size_t)y * c->w + x) * 8;
            for (int n = 0; n < 8; n++)
            {
                double s = 0.0;
                for (int t = 0; t < 9; t++) s += r[t] * (double)c->kl[n * 9 + t];
                o[n] = act_d(s + (double)c->bl[n], c->act, c->alpha_l, n);
            }
        }
}
static void d_l8_rows(void* p, int y0, int y1)
{
    d_ctx* c = (d_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            const double* rp[9];
            taps_d(c->in, c->w, x, y, c->h, rp);
            double s[8];
            conv8_d(rp, c->kl, c->bl, 8, s);
            size_t off = ((size_t)y * c->w + x) * 8;
            for (int n = 0; n < 8; n++)
            {
                double v = act_d(s[n], c->act, c->alpha_l, n);
                if (c->id) v = v * c->scale + c->id[off + n];
                c->out[off + n] = v;
            }
        }
}
static void d_deconv_rows(void* p, int y0, int y1)
{
    d_ctx* c = (d_ctx*)p;
    const float* k2 = c->k + 72 + 576 * 8;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            const double* rp[9];
            taps_d(c->in, c->w, x, y, c->h, rp);
            double s[8];
            conv8_d(rp, c->kl, c->bl, 8, s);
            for (int n = 0; n < 8; n++) s[n] = s[n] > 0.0 ? s[n] : 0.0;
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++)
                {
                    double d = 0.0;
                    for (int i = 0; i < 8; i++) d += s[i] * (double)k2[8 * (dy * 2 + dx) + i];
                    c->dst[(size_t)(2 * y + dy) * (2 * c->w) + 2 * x + dx] = d;
                }
        }
}
static void d_tail_rows(void* p, int y0, int y1)
{
    d_ctx* c = (d_ctx*)p;
    const int B = c->blocks;
    const float* k2 = c->k + 72 + 576 * (2 * B);
    const float* b2 = c->bi + 8 * (2 * B + 1);
    const float* a2 = c->al + 8 * B;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            const double* rp[9];
            taps_d(c->in, c->w, x, y, c->h, rp);
            size_t off = ((size_t)y * c->w + x) * 8;
            double buf[8];
            conv8_d(rp, c->kl, c->bl, 8, buf);
            for (int n = 0; n < 8; n++) buf[n] = buf[n] * c->scale + c->id[off + n];
            for (int n = 0; n < 8; n++)
            {
                double s = 0.0;
                for (int i = 0; i < 8; i++) s += buf[i] * (double)k2[n * 8 + i];
                s += (double)b2[n];
                s = s > 0.0 ? s : (double)a2[n] * s;
                c->out[off + n] = s + c->feat[off + n];
            }
        }
}
static void d_shuffle_rows(void* p, int y0, int y1)
{
    d_ctx* c = (d_ctx*)p;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            const double* rp[9];
            taps_d(c->in, c->w, x, y, c->h, rp);
            double s[4];
            conv8_d(rp, c->kl, c->bl, 4, s);
            double near = to_double(rowp(c->src, c->sstride, y), (size_t)x, c->type);
            for (int n = 0; n < 4; n++)
                c->dst[(size_t)(2 * y + (n >> 1)) * (2 * c->w) + 2 * x + (n & 1)] = s[n] + near;
        }
}

/* ACNetLegacy x2 in FP64; dst receives (2h)*(2w) unquantised, unsaturated doubles. */
int orc_acnet_legacy_x2_f64(const void* src, int w, int h, int sstride, int type,
                            double* dst, const float* kernels, const float* biases, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0) return -22;
    size_t n = (size_t)w * h * 8;
    double* a = (double*)malloc(n * sizeof(double));
    double* b = (double*)malloc(n * sizeof(double));
    if (!a || !b) { free(a); free(b); return -12; }
    d_ctx c;
    memset(&c, 0, sizeof(c));
    c.src = src; c.w = w; c.h = h; c.sstride = sstride; c.type = type; c.dst = dst; c.k = kernels; c.bi = biases;
    c.out = a; c.act = ACT_RELU; c.kl = kernels; c.bl = biases;
    parallel_rows(d_l0_rows, &c, h, threads);
    for (int l = 1; l < 8; l++)
    {
        c.in = a; c.out = b; c.kl = kernels + 72 + 576 * (l - 1); c.bl = biases + 8 * l; c.id = NULL;
        parallel_rows(d_l8_rows, &c, h, threads);
        double* t = a; a = b; b = t;
    }
    c.in = a; c.kl = kernels + 72 + 576 * 7; c.bl = biases + 64;
    parallel_rows(d_deconv_rows, &c, h, threads);
    free(a);
    free(b);
    return 0;
}

/* ARNet<8> x2 in FP64. */
int orc_arnet_x2_f64(const void* src, int w, int h, int sstride, int type,
                     double* dst, const float* kernels, const float* biases, const float* alphas,
                     int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 2) return -22;
    size_t n = (size_t)w * h * 8;
    double* feat = (double*)malloc(n * sizeof(double));
    double* t1 = (double*)malloc(n * sizeof(double));
    double* t2 = (double*)malloc(n * sizeof(double));
    double* t3 = (double*)malloc(n * sizeof(double));
    if (!feat || !t1 || !t2 || !t3) { free(feat); free(t1); free(t2); free(t3); return -12; }
    d_ctx c;
    memset(&c, 0, sizeof(c));
    c.src = src; c.w = w; c.h = h; c.sstride = sstride; c.type = type; c.dst = dst;
    c.k = kernels; c.bi = biases; c.al = alphas; c.blocks = blocks;
    int l = 0;
    c.out = feat; c.act = ACT_IDENTITY; c.kl = kernels; c.bl = biases;
    parallel_rows(d_l0_rows, &c, h, threads); l++;
#define KOFF(l) ((l) <= 0 ? 0 : 72 + 576 * ((l) - 1))
#define AOFF(l) (8 * (((l) - 1) / 2))
    c.in = feat; c.out = t1; c.act = ACT_PRELU; c.alpha_l = alphas + AOFF(l); c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = NULL;
    parallel_rows(d_l8_rows, &c, h, threads); l++;
    c.in = t1; c.out = t2; c.act = ACT_IDENTITY; c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = feat; c.scale = 0.2;
    parallel_rows(d_l8_rows, &c, h, threads); l++;
    for (int i = 0; i < blocks - 2; i++)
    {
        c.in = t2; c.out = t1; c.act = ACT_PRELU; c.alpha_l = alphas + AOFF(l); c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = NULL;
        parallel_rows(d_l8_rows, &c, h, threads); l++;
        c.in = t1; c.out = t3; c.act = ACT_IDENTITY; c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = t2; c.scale = 0.2;
        parallel_rows(d_l8_rows, &c, h, threads); l++;
        double* t = t2; t2 = t3; t3 = t;
    }
    c.in = t2; c.out = t1; c.act = ACT_PRELU; c.alpha_l = alphas + AOFF(l); c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = NULL;
    parallel_rows(d_l8_rows, &c, h, threads); l++;
    c.in = t1; c.out = t3; c.kl = kernels + KOFF(l); c.bl = biases + 8 * l; c.id = t2; c.scale = 0.2; c.feat = feat;
    parallel_rows(d_tail_rows, &c, h, threads); l += 2;
    c.in = t3; c.kl = kernels + 72 + 576 * (2 * blocks) + 64; c.bl = biases + 8 * l;
    parallel_rows(d_shuffle_rows, &c, h, threads);
#undef KOFF
#undef AOFF
    free(feat); free(t1); free(t2); free(t3);
    return 0;
}

/* ACNet<8> x2 in FP64. */
int orc_acnet8_x2_f64(const void* src, int w, int h, int sstride, int type,
                      double* dst, const float* kernels, const float* biases, const float* alphas,
                      int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || blocks < 1) return -22;
    size_t n = (size_t)w * h * 8;
    double* a = (double*)malloc(n * sizeof(double));
    double* b = (double*)malloc(n * sizeof(double));
    if (!a || !b) { free(a); free(b); return -12; }
    d_ctx c;
    memset(&c, 0, sizeof(c));
    c.src = src; c.w = w; c.h = h; c.sstride = sstride; c.type = type; c.dst = dst;
    c.k = kernels; c.bi = biases; c.al = alphas; c.blocks = blocks;
    c.out = a; c.act = ACT_PRELU; c.alpha_l = alphas; c.kl = kernels; c.bl = biases;
    parallel_rows(d_l0_rows, &c, h, threads);
    for (int l = 1; l <= blocks; l++)
    {
        c.in = a; c.out = b; c.act = ACT_PRELU; c.alpha_l = alphas + 8 * l;
        c.kl = kernels + 72 + 576 * (l - 1); c.bl = biases + 8 * l; c.id = NULL;
        parallel_rows(d_l8_rows, &c, h, threads);
        double* t = a; a = b; b = t;
    }
    c.in = a; c.kl = kernels + 72 + 576 * blocks; c.bl = biases + 8 * (blocks + 1);
    parallel_rows(d_shuffle_rows, &c, h, threads);
    free(a);
    free(b);
    return 0;
}

/* ----------------------------- FP64 twins of ArtCNN<F> and FSRCNNX<F> */

/* Same layer sequence as orc_artcnn_x2 / orc_fsrcnnx_x2, every map and sum in
 * double; dst receives the (2h) x (2w) unquantised, unsaturated output. */
typedef struct {
    const void* src; int w, h, sstride, type;
    const double* in; double* out; int cin, cout, K;
    const float* k; const float* b; int act; const float* alphas;
    const double* id;                  /* residual: out = act(conv) + id */
    const float* k2; const float* b2; const float* a2; const double* feat;  /* FSRCNNX tail */
    double* dst;
} gd_ctx;
static void gd_head_rows(void* p, int y0, int y1)
{
    gd_ctx* c = (gd_ctx*)p;
    const int K = c->K, R = K / 2;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            double r[25];
            for (int i = 0; i < K; i++)
            {
                int yy = y + i - R;
                yy = yy < 0 ? 0 : (yy > c->h - 1 ? c->h - 1 : yy);
                for (int j = 0; j < K; j++)
                {
                    int xx = x + j - R;
                    xx = xx < 0 ? 0 : (xx > c->w - 1 ? c->w - 1 : xx);
                    r[i * K + j] = to_double(rowp(c->src, c->sstride, yy), (size_t)xx, c->type);
                }
            }
            double* o = c->out + ((size_t)y * c->w + x) * c->cout;
            for (int n = 0; n < c->cout; n++)
            {
                double s = 0.0;
                for (int t = 0; t < K * K; t++) s += r[t] * (double)c->k[n * K * K + t];
                o[n] = act_d(s + (double)c->b[n], c->act, c->alphas, n);
            }
        }
}
static void gd_conv_sum(const gd_ctx* c, int x, int y, double* s)
{
    int xs[3], ys[3];
    taps3x3(x, y, c->w, c->h, xs, ys);
    for (int n = 0; n < c->cout; n++)
    {
        double acc = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
            {
                const double* rp = c->in + ((size_t)ys[i] * c->w + xs[j]) * c->cin;
                const float* kp = c->k + (size_t)n * c->cin * 9 + (size_t)(i * 3 + j) * c->cin;
                for (int ch = 0; ch < c->cin; ch++) acc += rp[ch] * (double)kp[ch];
            }
        s[n] = acc + (double)c->b[n];
    }
}
static void gd_conv_rows(void* p, int y0, int y1)
{
    gd_ctx* c = (gd_ctx*)p;
    double s[32];
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            gd_conv_sum(c, x, y, s);
            size_t off = ((size_t)y * c->w + x) * c->cout;
            for (int n = 0; n < c->cout; n++)
            {
                double v = act_d(s[n], c->act, c->alphas, n);
                if (c->id) v += c->id[off + n];
                c->out[off + n] = v;
            }
        }
}
static void gd_tail_rows(void* p, int y0, int y1)
{
    gd_ctx* c = (gd_ctx*)p;
    double s[32];
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            gd_conv_sum(c, x, y, s);
            for (int n = 0; n < c->cout; n++) s[n] = act_d(s[n], ACT_PRELU, c->alphas, n);
            size_t off = ((size_t)y * c->w + x) * c->cout;
            for (int n = 0; n < c->cout; n++)
            {
                double acc = 0.0;
                for (int i = 0; i < c->cout; i++) acc += s[i] * (double)c->k2[n * c->cout + i];
                acc += (double)c->b2[n] + c->feat[off + n];
                c->out[off + n] = act_d(acc, ACT_PRELU, c->a2, n);
            }
        }
}
static void gd_shuffle_rows(void* p, int y0, int y1)
{
    gd_ctx* c = (gd_ctx*)p;
    double s[4];
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < c->w; x++)
        {
            gd_conv_sum(c, x, y, s);
            for (int n = 0; n < 4; n++) c->dst[(size_t)(2 * y + (n >> 1)) * (2 * c->w) + 2 * x + (n & 1)] = s[n];
        }
}

/* family 1: ArtCNN<F> (orc_artcnn_x2's order), 2: FSRCNNX<F> (orc_fsrcnnx_x2's). */
int orc_f3_x2_f64(const void* src, int w, int h, int sstride, int type, double* dst, const float* kernels,
                  const float* biases, const float* alphas, int family, int F, int blocks, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || F < 1 || F > 32 || (family != 1 && family != 2)) return -22;
    if (family == 1 ? blocks < 1 : blocks < 2) return -22;
    size_t n = (size_t)w * h * F;
    double* feat = (double*)malloc(n * sizeof(double));
    double* a = (double*)malloc(n * sizeof(double));
    double* b = (double*)malloc(n * sizeof(double));
    if (!feat || !a || !b) { free(feat); free(a); free(b); return -12; }
    const int K = family == 1 ? 3 : 5;
    gd_ctx c;
    memset(&c, 0, sizeof(c));
    c.src = src; c.w = w; c.h = h; c.sstride = sstride; c.type = type; c.dst = dst;
    c.out = feat; c.cout = F; c.K = K; c.k = kernels; c.b = biases; c.act = ACT_IDENTITY;
    parallel_rows(gd_head_rows, &c, h, threads);
    const double* in = feat;
    const float* kl = kernels + F * K * K;
    int l = 1;
    c.cin = F; c.cout = F;
    if (family == 1)
    {
        for (int i = 0; i < blocks; i++, l++)
        {
            c.in = in; c.out = a; c.k = kl + (size_t)F * F * 9 * (l - 1); c.b = biases + F * l; c.act = ACT_RELU; c.id = NULL;
            parallel_rows(gd_conv_rows, &c, h, threads);
            in = a; double* t = a; a = b; b = t;
        }
        c.in = in; c.out = a; c.k = kl + (size_t)F * F * 9 * (l - 1); c.b = biases + F * l; c.act = ACT_IDENTITY; c.id = feat;
        parallel_rows(gd_conv_rows, &c, h, threads);
        in = a; l++;
        c.in = in; c.cout = 4; c.k = kl + (size_t)F * F * 9 * (l - 1); c.b = biases + F * l;
    }
    else
    {
        for (; l < blocks; l++)
        {
            c.in = in; c.out = a; c.k = kl + (size_t)F * F * 9 * (l - 1); c.b = biases + F * l; c.act = ACT_PRELU;
            c.alphas = alphas + F * (l - 1); c.id = NULL;
            parallel_rows(gd_conv_rows, &c, h, threads);
            in = a; double* t = a; a = b; b = t;
        }
        c.in = in; c.out = a; c.k = kl + (size_t)F * F * 9 * (l - 1); c.b = biases + F * l; c.alphas = alphas + F * (l - 1);
        c.k2 = kl + (size_t)F * F * 9 * blocks; c.b2 = biases + F * (l + 1); c.a2 = alphas + F * l; c.feat = feat;
        parallel_rows(gd_tail_rows, &c, h, threads);
        in = a; l += 2;
        c.in = in; c.cout = 4; c.k = kl + (size_t)F * F * 9 * blocks + F * F; c.b = biases + F * l;
    }
    parallel_rows(gd_shuffle_rows, &c, h, threads);
    free(feat); free(a); free(b);
    return 0;
}

/* ------------------------------------------------------ colour conversion */

/* rgb2yuv (ImageProcess.cpp:39-61) / rgba2yuva (:114-138): interleaved
 * RGB(A) in; planar Y (1 ch) and interleaved UV (2 ch) or UVA (3 ch) out,
 * all re-quantised to the source type. */
int orc_rgb2yuv(const void* rgb, int w, int h, int c, int sstride, int type,
                void* y, int ystride, void* uv, int uvstride)
{
    if (!rgb || !y || !uv || (c != 3 && c != 4)) return -22;
    for (int i = 0; i < h; i++)
    {
        const void* in = rowp(rgb, sstride, i);
        void* yo = rowpw(y, ystride, i);
        void* uo = rowpw(uv, uvstride, i);
        for (int j = 0; j < w; j++)
        {
            size_t base = (size_t)j * c;
            float r = to_float(in, base + 0, type);
            float g = to_float(in, base + 1, type);
            float b = to_float(in, base + 2, type);
            float a = 1.0f;
            if (c == 4)
            {
                a = to_float(in, base + 3, type);
                r = r * a; g = g * a; b = b * a;
            }
            float t0 = 0.299f * r, t1 = 0.587f * g, t2 = 0.114f * b;
            float yy = t0 + t1; yy = yy + t2;
            float u = 0.564f * (b - yy); u = u + 0.5f;
            float v = 0.713f * (r - yy); v = v + 0.5f;
            from_float(yo, (size_t)j, type, yy);
            int uc = c == 4 ? 3 : 2;
            from_float(uo, (size_t)j * uc + 0, type, u);
            from_float(uo, (size_t)j * uc + 1, type, v);
            if (c == 4) from_float(uo, (size_t)j * uc + 2, type, a);
        }
    }
    return 0;
}

/* yuv2rgb (ImageProcess.cpp:192-215) / yuva2rgba (:276-308). */
int orc_yuv2rgb(const void* y, int ystride, const void* uv, int uvstride, int w, int h, int c, int type,
                void* rgb, int dstride)
{
    if (!rgb || !y || !uv || (c != 3 && c != 4)) return -22;
    int uc = c == 4 ? 3 : 2;
    for (int i = 0; i < h; i++)
    {
        const void* yi = rowp(y, ystride, i);
        const void* ui = rowp(uv, uvstride, i);
        void* out = rowpw(rgb, dstride, i);
        for (int j = 0; j < w; j++)
        {
            float yy = to_float(yi, (size_t)j, type);
            float u = to_float(ui, (size_t)j * uc + 0, type) - 0.5f;
            float v = to_float(ui, (size_t)j * uc + 1, type) - 0.5f;
            float m0 = 1.403f * v;
            float r = yy + m0;
            float m1 = 0.344f * u, m2 = 0.714f * v;
            float g = yy - m1; g = g - m2;
            float m3 = 1.773f * u;
            float b = yy + m3;
            size_t base = (size_t)j * c;
            if (c == 4)
            {
                float a = to_float(ui, (size_t)j * uc + 2, type);
                if (a > 1e-6f) { r = r / a; g = g / a; b = b / a; }
                else r = g = b = 0.0f;
                from_float(out, base + 3, type, a);
            }
            from_float(out, base + 0, type, r);
            from_float(out, base + 1, type, g);
            from_float(out, base + 2, type, b);
        }
    }
    return 0;
}

/* --------------------------------------------------------------- resize */

/* Separable resampling restated from the filter definitions in
 * ImageResize.cpp:62-83 (bicubic b,c) and :127-134 (bilinear), with edge clamp
 * (ImageResize.cpp:269).  Sample placement: the centre of output pixel o maps
 * to source coordinate (o + 0.5) / scale - 0.5.  For downscaling the filter is
 * widened by 1/scale.  Weights are normalised to sum to 1.  Decode multiplies
 * by the reciprocal of the type's maximum; integer outputs are encoded with
 * fromFloat, float outputs are stored unsaturated.  Horizontal
 * pass first (float intermediate), then vertical; taps are summed in
 * ascending source order.  mode: 1 = Catmull-Rom, 16 = bilinear, 0 = point. */

static float filter_eval(int mode, float x)
{
    float ax = fabsf(x);
    if (mode == 16) return ax < 1.0f ? 1.0f - ax : 0.0f;
    if (mode == 0) return ax <= 0.5f ? 1.0f : 0.0f;
    /* Catmull-Rom: b = 0, c = 1/2. */
    if (ax < 1.0f) return 1.0f + ax * (0.0f + ax * (-2.5f + ax * 1.5f));
    if (ax < 2.0f) return 2.0f + ax * (-4.0f + ax * (2.5f + ax * -0.5f));
    return 0.0f;
}
static float filter_support(int mode) { return mode == 16 ? 1.0f : (mode == 0 ? 0.5f : 2.0f); }

/* Coefficient table: for each output index, first tap index (unclamped) and
 * up to maxtaps weights. Returns maxtaps. */
int orc_resize_coeffs(int n_in, int n_out, int mode, int* first, float* weights, int maxtaps)
{
    double scale = (double)n_out / (double)n_in;
    float sup = filter_support(mode);
    float fscale = scale < 1.0 ? (float)scale : 1.0f;
    float radius = sup / fscale;
    for (int o = 0; o < n_out; o++)
    {
        float center = (float)(((double)o + 0.5) / scale - 0.5);
        int lo = (int)ceilf(center - radius);
        int hi = (int)floorf(center + radius);
        if (mode == 0)
        {
            /* point: nearest source pixel (upscale) */
            lo = (int)floorf(center + 0.5f);
            hi = lo;
        }
        if (hi - lo + 1 > maxtaps) hi = lo + maxtaps - 1;
        float sum = 0.0f;
        float wv[64];
        int cnt = hi - lo + 1;
        for (int t = 0; t < cnt; t++)
        {
            float d = ((float)(lo + t) - center) * fscale;
            wv[t] = mode == 0 ? 1.0f : filter_eval(mode, d);
            sum += wv[t];
        }
        first[o] = lo;
        for (int t = 0; t < maxtaps; t++)
            weights[(size_t)o * maxtaps + t] = t < cnt ? (sum != 0.0f ? wv[t] / sum : 0.0f) : 0.0f;
    }
    return maxtaps;
}

static inline float decode(const void* base, size_t idx, int type)
{
    switch (type)
    {
    case ORC_U8: return (float)((const uint8_t*)base)[idx] * (1.0f / 255.0f);
    case ORC_U16: return (float)((const uint16_t*)base)[idx] * (1.0f / 65535.0f);
    default: return ((const float*)base)[idx];
    }
}

typedef struct {
    const void* src; int w, h, c, sstride, type;
    void* dst; int dw, dh, dstride;
    const int* fx; const int* fy; const float* wx; const float* wy; float* tmp; int mt; int stride;
} rs_ctx;

static void rs_h_rows(void* p, int y0, int y1)
{
    rs_ctx* k = (rs_ctx*)p;
    for (int i = y0; i < y1; i++)
    {
        const void* row = rowp(k->src, k->sstride, i);
        for (int o = 0; o < k->dw; o++)
            for (int ch = 0; ch < k->c; ch++)
            {
                float s = 0.0f;
                for (int t = 0; t < k->mt; t++)
                {
                    float wt = k->wx[(size_t)o * k->stride + t];
                    if (wt == 0.0f) continue;
                    int xi = k->fx[o] + t;
                    xi = xi < 0 ? 0 : (xi > k->w - 1 ? k->w - 1 : xi);
                    float m = wt * decode(row, (size_t)xi * k->c + ch, k->type);
                    s = s + m;
                }
                k->tmp[((size_t)i * k->dw + o) * k->c + ch] = s;
            }
    }
}

static void rs_v_rows(void* p, int o0, int o1)
{
    rs_ctx* k = (rs_ctx*)p;
    for (int o = o0; o < o1; o++)
    {
        void* row = rowpw(k->dst, k->dstride, o);
        for (int x = 0; x < k->dw; x++)
            for (int ch = 0; ch < k->c; ch++)
            {
                float s = 0.0f;
                for (int t = 0; t < k->mt; t++)
                {
                    float wt = k->wy[(size_t)o * k->stride + t];
                    if (wt == 0.0f) continue;
                    int yi = k->fy[o] + t;
                    yi = yi < 0 ? 0 : (yi > k->h - 1 ? k->h - 1 : yi);
                    float m = wt * k->tmp[((size_t)yi * k->dw + x) * k->c + ch];
                    s = s + m;
                }
                if (k->type == ORC_F32) ((float*)row)[(size_t)x * k->c + ch] = s; /* float output is not saturated */
                else from_float(row, (size_t)x * k->c + ch, k->type, s);
            }
    }
}

int orc_resize_mt(const void* src, int w, int h, int c, int sstride, int type,
                  void* dst, int dw, int dh, int dstride, int mode, int threads)
{
    if (!src || !dst || w <= 0 || h <= 0 || dw <= 0 || dh <= 0 || c <= 0) return -22;
    const int MT = 64;
    int* fx = (int*)malloc(sizeof(int) * dw);
    int* fy = (int*)malloc(sizeof(int) * dh);
    float* wx = (float*)malloc(sizeof(float) * dw * MT);
    float* wy = (float*)malloc(sizeof(float) * dh * MT);
    float* tmp = (float*)malloc(sizeof(float) * (size_t)h * dw * c);
    if (!fx || !fy || !wx || !wy || !tmp) { free(fx); free(fy); free(wx); free(wy); free(tmp); return -12; }
    orc_resize_coeffs(w, dw, mode, fx, wx, MT);
    orc_resize_coeffs(h, dh, mode, fy, wy, MT);
    /* trim the tap count to the widest non-zero span */
    int mt = 1;
    for (int o = 0; o < dw; o++) for (int t = 0; t < MT; t++) if (wx[(size_t)o * MT + t] != 0.0f && t + 1 > mt) mt = t + 1;
    for (int o = 0; o < dh; o++) for (int t = 0; t < MT; t++) if (wy[(size_t)o * MT + t] != 0.0f && t + 1 > mt) mt = t + 1;
    rs_ctx k = { src, w, h, c, sstride, type, dst, dw, dh, dstride, fx, fy, wx, wy, tmp, mt, MT };
    parallel_rows(rs_h_rows, &k, h, threads);   /* horizontal pass, float intermediate */
    parallel_rows(rs_v_rows, &k, dh, threads);  /* vertical pass */
    free(fx); free(fy); free(wx); free(wy); free(tmp);
    return 0;
}

int orc_resize(const void* src, int w, int h, int c, int sstride, int type,
               void* dst, int dw, int dh, int dstride, int mode)
{
    return orc_resize_mt(src, w, h, c, sstride, type, dst, dw, dh, dstride, mode, 1);
}

/* --------------------------------------------- synthetic ARNet parameters */

/* The reference's trained ARNet parameters are not available, so ARNet runs
 * use seeded synthetic parameters of the exact ARNet<8> shapes.  Generator:
 * splitmix64(seed) -> 24-bit uniform u in [-1, 1) -> u * scale (one float
 * multiply).  Order: every kernel layer in blob order, then biases, then
 * alphas.  The product library carries its own implementation of the same
 * generator; tests compare the two. */
static uint64_t sm64_next(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static float sm64_uniform(uint64_t* s)
{
    uint64_t r = sm64_next(s) >> 40; /* 24 bits */
    return (float)r * (1.0f / 8388608.0f) - 1.0f;
}
int orc_arnet_synth(int blocks, uint64_t seed, float* kernels, float* biases, float* alphas)
{
    if (blocks < 2) return -22;
    uint64_t s = seed;
    int nconv = 2 * blocks;
    int kl = 72 + 576 * nconv + 64 + 288;
    int bl = 8 + 8 * (nconv + 1) + 4;
    int al = 8 * (blocks + 1);
    for (int i = 0; i < kl; i++)
    {
        float scale;
        if (i < 72) scale = 0.5f;
        else if (i < 72 + 576 * nconv) scale = 0.12f;
        else if (i < 72 + 576 * nconv + 64) scale = 0.2f;
        else scale = 0.02f;
        kernels[i] = sm64_uniform(&s) * scale;
    }
    for (int i = 0; i < bl; i++) biases[i] = sm64_uniform(&s) * 0.01f;
    for (int i = 0; i < al; i++) alphas[i] = (sm64_uniform(&s) + 1.0f) * 0.125f;
    return 0;
}
