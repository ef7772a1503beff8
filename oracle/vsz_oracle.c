/*
 * vsz_oracle.c -- CPU restatement of vecSZ's dual-quantization compress/decompress path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU implementation is checked
 * against (tests/, __graft_entry__.smoke()) and the CPU baseline that bench.py times.  The product
 * (vecsz_gb300/) never links, loads or calls it.
 *
 * Every function restates one piece of the reference, in plain C, following the element-wise
 * rules the reference's AVX2 build actually executes (the AVX2 build is the reference's default
 * and the one its results are pinned to; its AVX-512 build does not compile,
 * src/dualquant.hh:135,142).  Citations are to files of szcompressor/vecSZ.
 *
 * Pinning: tests/test_oracle.py checks this file against tests/golden/ (fixtures produced by the
 * reference itself through oracle/ref/harness.cc) and, where oracle/_ref/libvszref.so could be
 * built (x86-64 only), against the reference directly on seeded random shapes.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).  No FMA contraction: the reference
 * computes every step as a separately rounded IEEE-754 operation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define VSO_OK 0
#define VSO_ERR_ARG 1
#define VSO_ERR_CORRUPT 3
#define VSO_ERR_CAPACITY 4

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------------------------ */
/* Error-bound family                                                                          */
/* ------------------------------------------------------------------------------------------ */

/* GetDatumValueRange<float> (src/types.cc:28-35): std::max_element / std::min_element (first
 * extreme under operator<), then the difference in float, widened to double on return. */
double vso_value_range(const float* d, size_t n) {
    if (n == 0) return 0.0;
    float mx = d[0], mn = d[0];
    for (size_t i = 1; i < n; i++) {
        if (mx < d[i]) mx = d[i];
        if (d[i] < mn) mn = d[i];
    }
    float r = mx - mn;
    return (double)r;
}

/* InitializeErrorBoundFamily (src/types.cc:84-92): {eb, 1/eb, 2eb, 1/(2eb)} in double. */
void vso_eb_family(double eb_final, double out[4]) {
    out[0] = eb_final;
    out[1] = 1 / eb_final;
    out[2] = 2 * eb_final;
    out[3] = 1 / (2 * eb_final);
}

/* ------------------------------------------------------------------------------------------ */
/* Prequantization and postquantization, one element at a time                                 */
/* ------------------------------------------------------------------------------------------ */

/* AVX prequant: _mm256_round_ps(_mm256_mul_ps(x, (float)(1/2eb)), NEAREST) -- an FP32 multiply
 * and round-half-to-even (src/dualquant.hh:89,290,622,784). */
static inline float pq_vec(float x, float r_f) {
    float p = x * r_f;
    return rintf(p);
}

/* Scalar prequant: round(data[id] * ebs_L4[EBx2_r]) -- a double multiply, round-half-away, then
 * stored into a float (src/dualquant.hh:109,298,631,796). */
static inline float pq_scalar(float x, double r_d) { return (float)round((double)x * r_d); }

/* AVX postquant (src/dualquant.hh:169-177,359-367,705-713): e = cur - pred; quantizable iff
 * sqrt(e*e) < R; code = cvtps_epi32(e + R) (round-to-even); outlier = andnot(q, cur). */
static inline void post_vec(float cur, float pred, float Rf, int32_t* code, float* outl) {
    float e  = cur - pred;
    float e2 = e * e;
    float ae = sqrtf(e2);
    if (ae < Rf) {
        *code = (int32_t)rintf(e + Rf);
        *outl = 0.0f;
    } else {
        *code = 0;
        *outl = cur;
    }
}

/* Scalar postquant (src/dualquant.hh:182-187,376-380,724-728): quantizable iff fabs(e) < R;
 * code = (int)(e + R) (truncation); outlier = (1 - q) * cur; code = q * code. */
static inline void post_scalar(float cur, float pred, int R, int32_t* code, float* outl) {
    float e = cur - pred;
    int q   = fabsf(e) < (float)R;
    *code   = q ? (int32_t)(e + (float)R) : 0;
    *outl   = (float)(1 - q) * cur;
}

/* ------------------------------------------------------------------------------------------ */
/* Padding (-p): the value(s) that replace the zero halo of each Lorenzo block.                */
/* src/utils/padding.hh (find_pad_value :122-143, find_edge_pad_value :145-207, block_pad       */
/* :209-254, edge_pad :256-301, x_block_pad / x_edge_pad :303-373); call sites                  */
/* src/vecsz_interface.hh:70-90 (global value, pad array sizes) and src/dualquant.hh:36-46,     */
/* 224-246, 551-573 (compress), 916-1016 (decompress).                                          */
/*                                                                                              */
/* Rules (each one what the single-threaded reference computes):                                */
/*  - Block grid: get_nblk = (d + bs + 1) / bs per axis (src/dimensions.hh:32), phantom blocks   */
/*    past the field included; pad values are stored block by block, x fastest.                 */
/*  - global: p = find_pad_value over the whole field; the archive holds                         */
/*    (float)round((double)p * r_d) (interface:79); 1D predicts from that value, 2D/3D from      */
/*    roundf((float)((double)p * r_d)) (block_pad's float multiply then round, padding.hh:219).  */
/*  - block: one value per block.  1D: find_pad_value over the block's bs raw values, NOT        */
/*    prequantized (dualquant.hh:40).  2D/3D: over the block's cells (x fastest), then           */
/*    roundf((float)((double)v * r_d)).                                                          */
/*  - edge: 1D as block.  2D: [top row y=0, left column x=0]; 3D: [front face z=0 (x, y),        */
/*    left face x=0 (y, z), top face y=0 (x, z)], each prequantized like block values.           */
/*    The halo takes them as (padding.hh:286-296): 2D x-halo (and corner) = v0, y-halo = v1;     */
/*    3D z-halo plane = v0, y-halo = v1, x-halo = v2.                                             */
/*  - max / min: m = v[0]; m = v[i] > m ? v[i] : m (first maximum wins; a leading NaN sticks).    */
/*    avg: float running sum in order, divided by (float)count.  constant: the given value.      */
/*  - Cells outside the field count as 0.0f.  The reference reads memory past the field there    */
/*    (1D) or an uninitialised buffer (2D/3D fill_*_block); zeros are what it computes when that  */
/*    memory is zero.                                                                             */
/* ------------------------------------------------------------------------------------------ */

#define VSO_PAD_NONE 0
#define VSO_PAD_GLOBAL 1
#define VSO_PAD_BLOCK 2
#define VSO_PAD_EDGE 3
#define VSO_PADV_MAX 0
#define VSO_PADV_MIN 1
#define VSO_PADV_AVG 2
#define VSO_PADV_CONST 3

static size_t nblk_of(size_t d, int bs) { return (d + (size_t)bs + 1) / (size_t)bs; }

/* find_pad_value (padding.hh:122-143) over n values in visiting order. */
static float find_pad(const float* v, size_t n, int type, float cst) {
    if (type == VSO_PADV_CONST) return cst;
    if (type == VSO_PADV_AVG) {
        float s = 0.0f;
        for (size_t i = 0; i < n; i++) s += v[i];
        return s / (float)n;
    }
    float m = v[0];
    for (size_t i = 0; i < n; i++) {
        if (type == VSO_PADV_MAX) m = (v[i] > m) ? v[i] : m;
        else m = (v[i] < m) ? v[i] : m;
    }
    return m;
}

static float field_at(const float* x, size_t d0, size_t d1, size_t d2, size_t g0, size_t g1, size_t g2) {
    return (g0 < d0 && g1 < d1 && g2 < d2) ? x[g0 + d0 * (g1 + d1 * g2)] : 0.0f;
}

static float prequant_pad(float v, double r_d) {
    float t = (float)((double)v * r_d); /* padValueLocal *= padValueModifier */
    return roundf(t);
}

/* Number of pad values an archive of this geometry holds (interface:78-89). */
size_t vso_pad_count(int ndim, size_t d0, size_t d1, size_t d2, int bs, int mode) {
    size_t nb = nblk_of(d0, bs) * nblk_of(d1, bs) * nblk_of(d2, bs);
    if (mode == VSO_PAD_GLOBAL) return 1;
    if (mode == VSO_PAD_BLOCK) return nb;
    if (mode == VSO_PAD_EDGE) return (ndim == 1 ? 1 : (size_t)ndim) * nb;
    return 0;
}

/* Pad values: arch[vso_pad_count] as the archive stores them; *halo_global: the value the
 * compressor predicts from in global mode. */
int vso_pad_values(const float* x, int ndim, size_t d0, size_t d1, size_t d2, int bs, int mode, int type, float cst,
                   double r_d, float* arch, float* halo_global) {
    if (mode < VSO_PAD_NONE || mode > VSO_PAD_EDGE || type < VSO_PADV_MAX || type > VSO_PADV_CONST) return VSO_ERR_ARG;
    if (halo_global) *halo_global = 0.0f;
    if (mode == VSO_PAD_NONE) return VSO_OK;
    if (mode == VSO_PAD_GLOBAL) {
        float p    = find_pad(x, d0 * d1 * d2, type, cst);
        arch[0]    = (float)round((double)p * r_d);
        if (halo_global) *halo_global = (ndim == 1) ? arch[0] : prequant_pad(p, r_d);
        return VSO_OK;
    }
    size_t nb0 = nblk_of(d0, bs), nb1 = nblk_of(d1, bs), nb2 = nblk_of(d2, bs);
    size_t cells = (size_t)bs * (ndim >= 2 ? (size_t)bs : 1) * (ndim == 3 ? (size_t)bs : 1);
    float* buf   = (float*)malloc(sizeof(float) * cells);
    if (!buf) return VSO_ERR_ARG;
    size_t k = 0;
    for (size_t b2 = 0; b2 < nb2; b2++)
        for (size_t b1 = 0; b1 < nb1; b1++)
            for (size_t b0 = 0; b0 < nb0; b0++) {
                size_t o0 = b0 * bs, o1 = b1 * bs, o2 = b2 * bs;
                if (ndim == 1) {
                    for (int i = 0; i < bs; i++) buf[i] = field_at(x, d0, d1, d2, o0 + i, 0, 0);
                    arch[k++] = find_pad(buf, (size_t)bs, type, cst);
                } else if (mode == VSO_PAD_BLOCK) {
                    size_t c = 0;
                    for (int j3 = 0; j3 < (ndim == 3 ? bs : 1); j3++)
                        for (int j = 0; j < bs; j++)
                            for (int i = 0; i < bs; i++) buf[c++] = field_at(x, d0, d1, d2, o0 + i, o1 + j, o2 + j3);
                    arch[k++] = prequant_pad(find_pad(buf, cells, type, cst), r_d);
                } else if (ndim == 2) {
                    for (int i = 0; i < bs; i++) buf[i] = field_at(x, d0, d1, d2, o0 + i, o1, 0);
                    arch[k++] = prequant_pad(find_pad(buf, (size_t)bs, type, cst), r_d);
                    for (int i = 0; i < bs; i++) buf[i] = field_at(x, d0, d1, d2, o0, o1 + i, 0);
                    arch[k++] = prequant_pad(find_pad(buf, (size_t)bs, type, cst), r_d);
                } else {
                    size_t f = (size_t)bs * bs;
                    for (int j = 0; j < bs; j++)
                        for (int i = 0; i < bs; i++) buf[i + j * bs] = field_at(x, d0, d1, d2, o0 + i, o1 + j, o2);
                    arch[k++] = prequant_pad(find_pad(buf, f, type, cst), r_d);
                    for (int j = 0; j < bs; j++)
                        for (int i = 0; i < bs; i++) buf[i + j * bs] = field_at(x, d0, d1, d2, o0, o1 + i, o2 + j);
                    arch[k++] = prequant_pad(find_pad(buf, f, type, cst), r_d);
                    for (int j = 0; j < bs; j++)
                        for (int i = 0; i < bs; i++) buf[i + j * bs] = field_at(x, d0, d1, d2, o0 + i, o1, o2 + j);
                    arch[k++] = prequant_pad(find_pad(buf, f, type, cst), r_d);
                }
            }
    free(buf);
    return VSO_OK;
}

/* Halo values of block `blk` (pv[0..2], see the rules above).  mode: how the pad array is read --
 * NONE (zero halo), GLOBAL (hg for every block), BLOCK (arch[blk]) or EDGE (ndim values). */
static void block_halo(int ndim, int mode, const float* arch, float hg, size_t blk, float pv[3]) {
    pv[0] = pv[1] = pv[2] = 0.0f;
    if (mode == VSO_PAD_GLOBAL) pv[0] = pv[1] = pv[2] = hg;
    else if (mode == VSO_PAD_BLOCK || (mode == VSO_PAD_EDGE && ndim == 1)) pv[0] = pv[1] = pv[2] = arch[blk];
    else if (mode == VSO_PAD_EDGE)
        for (int i = 0; i < ndim; i++) pv[i] = arch[(size_t)ndim * blk + (size_t)i];
}

/* x_block_pad / x_edge_pad layout of the (bs+1)^ndim block buffer (padding.hh:303-373). */
static void fill_halo2(float* s, int W, const float pv[3]) {
    memset(s, 0, sizeof(float) * (size_t)W * W);
    for (int j = 0; j < W; j++)
        for (int i = 0; i < W; i++)
            if (i == 0) s[j * W + i] = pv[0];
            else if (j == 0) s[j * W + i] = pv[1];
}

static void fill_halo3(float* s, int W, const float pv[3]) {
    memset(s, 0, sizeof(float) * (size_t)W * W * W);
    for (int k = 0; k < W; k++)
        for (int j = 0; j < W; j++)
            for (int i = 0; i < W; i++) {
                float* c = &s[((size_t)k * W + j) * W + i];
                if (k == 0) *c = pv[0];
                else if (j == 0) *c = pv[1];
                else if (i == 0) *c = pv[2];
            }
}

/* ------------------------------------------------------------------------------------------ */
/* c_lorenzo_{1,2,3}d1l, all blocks (src/dualquant.hh:19-913; driven by                        */
/* src/vecsz_interface.hh:108-140).  Outputs are dense like the reference's `code`/`outlier`    */
/* arrays: code[i] in [0, 2R), outlier[i] = prequantized value where code[i] == 0, else 0.      */
/* Block counts follow get_nblk = (d + bs + 1) / bs (src/dimensions.hh:32); blocks wholly       */
/* outside the field touch nothing.  Requires bs to be a positive multiple of 8.               */
/* pmode / arch / hg: the halo (block_halo); VSO_PAD_NONE is the reference's zero halo.        */
/* ------------------------------------------------------------------------------------------ */

static void lorenzo_1d(const float* x, size_t d0, int bs, int R, double r_d, int32_t* code, float* outl, int pmode,
                       const float* arch, float hg) {
    const float r_f = (float)r_d, Rf = (float)R;
    long nblk       = (long)((d0 + bs + 1) / bs);
    (void)r_d;
#pragma omp parallel for schedule(static)
    for (long b0 = 0; b0 < nblk; b0++) {
        size_t o = (size_t)b0 * bs;
        if (o >= d0) continue;
        /* Prequant runs on whole 8-wide AVX chunks (blocks start on multiples of 8), the
         * postquant on AVX chunks for blocks with o + bs < d0, scalar otherwise; the two postquant
         * forms agree on integer-valued residuals (src/dualquant.hh:65-205) -- and differ on the
         * first element of a block padded with a raw, non-integer value (:155-187). */
        int full  = o + bs < d0;
        float pv[3];
        block_halo(1, pmode, arch, hg, (size_t)b0, pv);
        float prev = pv[0]; /* the block's padding (0 without -p) */
        for (int k = 0; k < bs; k++) {
            size_t g = o + k;
            if (g >= d0) break;
            float s = pq_vec(x[g], r_f);
            if (full) post_vec(s, prev, Rf, &code[g], &outl[g]);
            else post_scalar(s, prev, R, &code[g], &outl[g]);
            prev = s;
        }
    }
}

static void lorenzo_2d(const float* x, size_t d0, size_t d1, int bs, int R, double r_d, int32_t* code,
                       float* outl, int pmode, const float* arch, float hg) {
    const float r_f = (float)r_d, Rf = (float)R;
    long nb0 = (long)((d0 + bs + 1) / bs), nb1 = (long)((d1 + bs + 1) / bs);
    const int W = bs + 1;
#pragma omp parallel
    {
        float* s = (float*)malloc(sizeof(float) * W * W);
#pragma omp for schedule(static)
        for (long b1 = 0; b1 < nb1; b1++) {
            for (long b0 = 0; b0 < nb0; b0++) {
                size_t o0 = (size_t)b0 * bs, o1 = (size_t)b1 * bs;
                if (o0 >= d0 || o1 >= d1) continue;
                float pv[3];
                block_halo(2, pmode, arch, hg, (size_t)b0 + (size_t)nb0 * (size_t)b1, pv);
                fill_halo2(s, W, pv);
                int interior = (o1 + bs < d1) && (o0 + bs < d0); /* src/dualquant.hh:252 */
                /* Prequant: every cell of the block goes through the AVX form, edge blocks too
                 * (src/dualquant.hh:268-292,400-424); cells outside the field never feed an
                 * in-range residual, so they stay 0 here. */
                for (int i1 = 0; i1 < bs; i1++)
                    for (int i0 = 0; i0 < bs; i0++) {
                        size_t g0 = o0 + i0, g1 = o1 + i1;
                        if (g0 < d0 && g1 < d1) s[(i1 + 1) * W + (i0 + 1)] = pq_vec(x[g0 + g1 * d0], r_f);
                    }
                for (int i1 = 0; i1 < bs; i1++) {
                    size_t g1 = o1 + i1;
                    if (g1 >= d1) continue;
                    for (int i0 = 0; i0 < bs; i0++) {
                        size_t g0 = o0 + i0;
                        if (g0 >= d0) continue;
                        size_t id = g0 + g1 * d0;
                        /* Edge blocks skip (`continue`) every AVX chunk that is not wholly inside
                         * the field and never run the scalar tail, so those elements keep the
                         * zero-initialised code 0 / outlier 0 (src/dualquant.hh:490-495). */
                        int chunk0 = i0 & ~7;
                        if (!interior && o0 + chunk0 + 7 >= d0) {
                            code[id] = 0;
                            outl[id] = 0.0f;
                            continue;
                        }
                        float W_ = s[(i1 + 1) * W + i0], N_ = s[i1 * W + (i0 + 1)], NW = s[i1 * W + i0];
                        float cur  = s[(i1 + 1) * W + (i0 + 1)];
                        float pred = W_ + (N_ - NW); /* src/dualquant.hh:358,502 */
                        post_vec(cur, pred, Rf, &code[id], &outl[id]);
                    }
                }
            }
        }
        free(s);
    }
}

#define S3(z, y, x) s[((z) * W + (y)) * W + (x)]

static void lorenzo_3d(const float* x, size_t d0, size_t d1, size_t d2, int bs, int R, double r_d, int32_t* code,
                       float* outl, int pmode, const float* arch, float hg) {
    const float r_f = (float)r_d, Rf = (float)R;
    long nb0 = (long)((d0 + bs + 1) / bs), nb1 = (long)((d1 + bs + 1) / bs), nb2 = (long)((d2 + bs + 1) / bs);
    const int W = bs + 1;
#pragma omp parallel
    {
        float* s = (float*)malloc(sizeof(float) * W * W * W);
#pragma omp for schedule(static)
        for (long b2 = 0; b2 < nb2; b2++) {
            for (long b1 = 0; b1 < nb1; b1++) {
                for (long b0 = 0; b0 < nb0; b0++) {
                    size_t o0 = (size_t)b0 * bs, o1 = (size_t)b1 * bs, o2 = (size_t)b2 * bs;
                    if (o0 >= d0 || o1 >= d1 || o2 >= d2) continue;
                    float pv[3];
                    block_halo(3, pmode, arch, hg, (size_t)b0 + (size_t)nb0 * ((size_t)b1 + (size_t)nb1 * (size_t)b2), pv);
                    fill_halo3(s, W, pv);
                    int interior = (o2 + bs < d2) && (o1 + bs < d1) && (o0 + bs < d0); /* :580 */
                    /* Number of leading AVX elements in each in-range row: interior blocks are all
                     * AVX; edge blocks run 8-wide chunks until the first chunk that is not wholly
                     * inside the field (`break`), and the scalar loop takes the rest of the row
                     * (src/dualquant.hh:776-797, 863-908). */
                    int navx = bs;
                    if (!interior) {
                        navx = 0;
                        while (navx < bs && o0 + navx + 7 < d0) navx += 8;
                    }
                    for (int i2 = 0; i2 < bs; i2++)
                        for (int i1 = 0; i1 < bs; i1++)
                            for (int i0 = 0; i0 < bs; i0++) {
                                size_t g0 = o0 + i0, g1 = o1 + i1, g2 = o2 + i2;
                                if (g0 >= d0 || g1 >= d1 || g2 >= d2) continue;
                                float v = x[g0 + g1 * d0 + g2 * d0 * d1];
                                S3(i2 + 1, i1 + 1, i0 + 1) = (i0 < navx) ? pq_vec(v, r_f) : pq_scalar(v, r_d);
                            }
                    for (int i2 = 0; i2 < bs; i2++)
                        for (int i1 = 0; i1 < bs; i1++)
                            for (int i0 = 0; i0 < bs; i0++) {
                                size_t g0 = o0 + i0, g1 = o1 + i1, g2 = o2 + i2;
                                if (g0 >= d0 || g1 >= d1 || g2 >= d2) continue;
                                size_t id  = g0 + g1 * d0 + g2 * d0 * d1;
                                float XYZ  = S3(i2, i1, i0);
                                float XY   = S3(i2 + 1, i1, i0);
                                float XZ   = S3(i2, i1 + 1, i0);
                                float YZ   = S3(i2, i1, i0 + 1);
                                float X    = S3(i2 + 1, i1 + 1, i0);
                                float Y    = S3(i2 + 1, i1, i0 + 1);
                                float Z    = S3(i2, i1 + 1, i0 + 1);
                                float cur  = S3(i2 + 1, i1 + 1, i0 + 1);
                                if (i0 < navx) {
                                    /* src/dualquant.hh:702-704 */
                                    float dist1 = X + (Y + Z);
                                    float dist2 = XY + (XZ + YZ);
                                    float pred  = (XYZ - dist2) + dist1;
                                    post_vec(cur, pred, Rf, &code[id], &outl[id]);
                                } else {
                                    /* src/dualquant.hh:900-902, evaluated left to right */
                                    float pred = XYZ - XY - XZ - YZ + X + Y + Z;
                                    post_scalar(cur, pred, R, &code[id], &outl[id]);
                                }
                            }
                }
            }
        }
        free(s);
    }
}

/* Dual-quant compress over the whole field.  code/outlier are written for every element. */
int vso_dualquant(const float* x, int ndim, size_t d0, size_t d1, size_t d2, int bs, int radius, double ebx2_r,
                  int32_t* code, float* outlier) {
    if (bs <= 0 || bs % 8) return VSO_ERR_ARG;
    if (ndim == 1) lorenzo_1d(x, d0, bs, radius, ebx2_r, code, outlier, VSO_PAD_NONE, NULL, 0.0f);
    else if (ndim == 2) lorenzo_2d(x, d0, d1, bs, radius, ebx2_r, code, outlier, VSO_PAD_NONE, NULL, 0.0f);
    else if (ndim == 3) lorenzo_3d(x, d0, d1, d2, bs, radius, ebx2_r, code, outlier, VSO_PAD_NONE, NULL, 0.0f);
    else return VSO_ERR_ARG;
    return VSO_OK;
}

/* Dual-quant compress with padding: the pad values (vso_pad_values) are computed first, then every
 * block predicts from its halo.  pad_out: vso_pad_count floats, the archive's pad section. */
int vso_dualquant_pad(const float* x, int ndim, size_t d0, size_t d1, size_t d2, int bs, int radius, double ebx2_r,
                      int pad_mode, int pad_type, float pad_const, int32_t* code, float* outlier, float* pad_out) {
    if (bs <= 0 || bs % 8) return VSO_ERR_ARG;
    float hg = 0.0f;
    int rc   = vso_pad_values(x, ndim, d0, d1, d2, bs, pad_mode, pad_type, pad_const, ebx2_r, pad_out, &hg);
    if (rc) return rc;
    if (ndim == 1) lorenzo_1d(x, d0, bs, radius, ebx2_r, code, outlier, pad_mode, pad_out, hg);
    else if (ndim == 2) lorenzo_2d(x, d0, d1, bs, radius, ebx2_r, code, outlier, pad_mode, pad_out, hg);
    else if (ndim == 3) lorenzo_3d(x, d0, d1, d2, bs, radius, ebx2_r, code, outlier, pad_mode, pad_out, hg);
    else return VSO_ERR_ARG;
    return VSO_OK;
}

/* Outlier gather (src/vecsz_interface.hh:166-170): values where code == 0, in index order. */
size_t vso_gather_outliers(const int32_t* code, const float* outlier, size_t n, float* out) {
    size_t k = 0;
    for (size_t i = 0; i < n; i++)
        if (code[i] == 0) out[k++] = outlier[i];
    return k;
}

/* Outlier scatter (src/vecsz_interface.hh:313-317). */
size_t vso_scatter_outliers(const int32_t* code, const float* outliers, size_t n, float* outlier_dense) {
    size_t k = 0;
    for (size_t i = 0; i < n; i++) outlier_dense[i] = (code[i] == 0) ? outliers[k++] : 0.0f;
    return k;
}

/* ------------------------------------------------------------------------------------------ */
/* x_lorenzo_{1,2,3}d1l (src/dualquant.hh:915-1043; driven by src/vecsz_interface.hh:323-354).   */
/* s = code == 0 ? outlier : (float)(pred + (code - R)); xhat = (float)((double)s * 2eb).       */
/* ------------------------------------------------------------------------------------------ */

/* How a decompressor reads n_pad values (src/vecsz_interface.hh:287-298): 1 -> global, one per
 * block -> block, ndim per block -> edge, otherwise no padding (zero halo; 1D then reads pad[0]
 * for every block, dualquant.hh:924-927, and 0 when the section is empty). */
static int pad_mode_of(size_t npad, int ndim, size_t nb) {
    if (npad == 1) return VSO_PAD_GLOBAL;
    if (npad == nb) return VSO_PAD_BLOCK;
    if (npad == (size_t)ndim * nb) return VSO_PAD_EDGE;
    return VSO_PAD_NONE;
}

int vso_xlorenzo_pad(const int32_t* code, const float* outlier, int ndim, size_t d0, size_t d1, size_t d2, int bs,
                     int radius, double ebx2, const float* pads, size_t npad, float* xhat) {
    if (bs <= 0) return VSO_ERR_ARG;
    const int R = radius;
    long nb0 = (long)nblk_of(d0, bs), nb1 = (long)nblk_of(d1, bs), nb2 = (long)nblk_of(d2, bs);
    int pmode = pad_mode_of(npad, ndim, (size_t)nb0 * nb1 * nb2);
    if (ndim == 1) {
#pragma omp parallel for schedule(static)
        for (long b0 = 0; b0 < nb0; b0++) {
            size_t o = (size_t)b0 * bs;
            /* block / edge: pad[b0]; otherwise pad[0] (0 for an empty pad section: the reference
             * reads pad_vals[0] from an empty array there) */
            float pad = 0.0f;
            if (pmode == VSO_PAD_BLOCK || pmode == VSO_PAD_EDGE) pad = pads[b0];
            else if (npad > 0) pad = pads[0];
            for (int i0 = 0; i0 < bs; i0++) {
                size_t id = o + i0;
                if (id >= d0) continue;
                float pred = (id < o + 1) ? pad : xhat[id - 1];
                xhat[id]   = code[id] == 0 ? outlier[id] : (float)(pred + (float)(code[id] - R));
            }
            for (int i0 = 0; i0 < bs; i0++) {
                size_t id = o + i0;
                if (id >= d0) continue;
                xhat[id] = (float)((double)xhat[id] * ebx2);
            }
        }
        return VSO_OK;
    }
    const int W = bs + 1;
    const float hg = (pmode == VSO_PAD_GLOBAL) ? pads[0] : 0.0f;
    if (ndim == 2) {
#pragma omp parallel
        {
            float* s = (float*)malloc(sizeof(float) * W * W);
#pragma omp for schedule(static)
            for (long b1 = 0; b1 < nb1; b1++)
                for (long b0 = 0; b0 < nb0; b0++) {
                    float pv[3];
                    block_halo(2, pmode, pads, hg, (size_t)b0 + (size_t)nb0 * b1, pv);
                    fill_halo2(s, W, pv);
                    size_t o0 = (size_t)b0 * bs, o1 = (size_t)b1 * bs;
                    for (int i1 = 0; i1 < bs; i1++)
                        for (int i0 = 0; i0 < bs; i0++) {
                            size_t g0 = o0 + i0, g1 = o1 + i1;
                            if (g1 >= d1 || g0 >= d0) continue;
                            size_t id  = g0 + g1 * d0;
                            float pred = s[i1 * W + (i0 + 1)] + s[(i1 + 1) * W + i0] - s[i1 * W + i0];
                            float v    = code[id] == 0 ? outlier[id] : (float)(pred + (float)(code[id] - R));
                            s[(i1 + 1) * W + (i0 + 1)] = v;
                            xhat[id]                   = (float)((double)v * ebx2);
                        }
                }
            free(s);
        }
        return VSO_OK;
    }
    if (ndim == 3) {
#pragma omp parallel
        {
            float* s = (float*)malloc(sizeof(float) * W * W * W);
#pragma omp for schedule(static)
            for (long b2 = 0; b2 < nb2; b2++)
                for (long b1 = 0; b1 < nb1; b1++)
                    for (long b0 = 0; b0 < nb0; b0++) {
                        float pv[3];
                        block_halo(3, pmode, pads, hg, (size_t)b0 + (size_t)nb0 * ((size_t)b1 + (size_t)nb1 * b2), pv);
                        fill_halo3(s, W, pv);
                        size_t o0 = (size_t)b0 * bs, o1 = (size_t)b1 * bs, o2 = (size_t)b2 * bs;
                        for (int i2 = 0; i2 < bs; i2++)
                            for (int i1 = 0; i1 < bs; i1++)
                                for (int i0 = 0; i0 < bs; i0++) {
                                    size_t g0 = o0 + i0, g1 = o1 + i1, g2 = o2 + i2;
                                    if (g2 >= d2 || g1 >= d1 || g0 >= d0) continue;
                                    size_t id  = g0 + g1 * d0 + g2 * d1 * d0;
                                    float pred = S3(i2, i1, i0) - S3(i2 + 1, i1, i0) - S3(i2, i1 + 1, i0) -
                                                 S3(i2, i1, i0 + 1) + S3(i2 + 1, i1 + 1, i0) +
                                                 S3(i2 + 1, i1, i0 + 1) + S3(i2, i1 + 1, i0 + 1);
                                    float v = code[id] == 0 ? outlier[id] : (float)(pred + (float)(code[id] - R));
                                    S3(i2 + 1, i1 + 1, i0 + 1) = v;
                                    xhat[id]                   = (float)((double)v * ebx2);
                                }
                    }
            free(s);
        }
        return VSO_OK;
    }
    return VSO_ERR_ARG;
}

int vso_xlorenzo(const int32_t* code, const float* outlier, int ndim, size_t d0, size_t d1, size_t d2, int bs,
                 int radius, double ebx2, float* xhat) {
    return vso_xlorenzo_pad(code, outlier, ndim, d0, d1, d2, bs, radius, ebx2, NULL, 0, xhat);
}

/* ------------------------------------------------------------------------------------------ */
/* Tree Huffman (src/huffman.hh).  The tree is built with the reference's own binary-heap       */
/* priority queue (qinsert :169-177, qremove :179-192); its removal places the last heap entry  */
/* at the leaf the hole sank to without sifting it up, so the "heap" is not always ordered and  */
/* only an operation-for-operation replay gives the same tree.                                  */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    int32_t left, right; /* -1: none */
    uint64_t freq;
    uint8_t t; /* 1 leaf, 0 internal */
    uint32_t c;
} vso_node;

typedef struct {
    uint32_t state_num, all_nodes;
    vso_node* pool;
    int n_nodes;
    int32_t* qq; /* 1-based heap of pool indices */
    int qend;
    uint8_t* cout;      /* code length per symbol */
    uint64_t* code0;    /* first 64 bits of the left-aligned codeword */
    uint64_t* code1;    /* next 64 bits (codes longer than 64) */
    uint8_t* has_code;
    int n_inode;
} vso_tree;

/* createHuffmanTree (src/huffman.hh:116-137) */
static vso_tree* tree_create(int state_num) {
    vso_tree* h  = (vso_tree*)calloc(1, sizeof(vso_tree));
    h->state_num = (uint32_t)state_num;
    h->all_nodes = 2u * (uint32_t)state_num;
    h->pool      = (vso_node*)calloc((size_t)h->all_nodes * 2, sizeof(vso_node));
    h->qq        = (int32_t*)calloc((size_t)h->all_nodes * 2 + 2, sizeof(int32_t));
    h->cout      = (uint8_t*)calloc(h->state_num, 1);
    h->code0     = (uint64_t*)calloc(h->state_num, 8);
    h->code1     = (uint64_t*)calloc(h->state_num, 8);
    h->has_code  = (uint8_t*)calloc(h->state_num, 1);
    h->qend      = 1;
    return h;
}

static void tree_free(vso_tree* h) {
    if (!h) return;
    free(h->pool);
    free(h->qq);
    free(h->cout);
    free(h->code0);
    free(h->code1);
    free(h->has_code);
    free(h);
}

/* new_node (src/huffman.hh:146-160) */
static int new_leaf(vso_tree* h, uint64_t freq, uint32_t c) {
    int n         = h->n_nodes++;
    vso_node* p   = &h->pool[n];
    p->c          = c;
    p->freq       = freq;
    p->t          = 1;
    p->left       = -1;
    p->right      = -1;
    return n;
}

static int new_internal(vso_tree* h, int a, int b) {
    int n       = h->n_nodes++;
    vso_node* p = &h->pool[n];
    p->left     = a;
    p->right    = b;
    p->freq     = h->pool[a].freq + h->pool[b].freq;
    p->t        = 0;
    p->c        = 0;
    return n;
}

/* qinsert (src/huffman.hh:169-177) */
static void qinsert(vso_tree* h, int n) {
    int j, i = h->qend++;
    while ((j = (i >> 1))) {
        if (h->pool[h->qq[j]].freq <= h->pool[n].freq) break;
        h->qq[i] = h->qq[j];
        i        = j;
    }
    h->qq[i] = n;
}

/* qremove (src/huffman.hh:179-192) */
static int qremove(vso_tree* h) {
    int i = 1, l;
    int n = h->qq[i];
    if (h->qend < 2) return -1;
    h->qend--;
    while ((l = (i << 1)) < h->qend) {
        if (l + 1 < h->qend && h->pool[h->qq[l + 1]].freq < h->pool[h->qq[l]].freq) l++;
        h->qq[i] = h->qq[l];
        i        = l;
    }
    h->qq[i] = h->qq[h->qend];
    return n;
}

/* build_code (src/huffman.hh:200-227): left edge 0, right edge 1; codewords left-aligned in two
 * 64-bit words.  A one-leaf tree gets length 0 and codeword 0. */
static void build_code(vso_tree* h, int n, int len, uint64_t out1, uint64_t out2) {
    vso_node* p = &h->pool[n];
    if (p->t) {
        if (len <= 64) {
            h->code0[p->c] = (len == 0) ? 0 : (out1 << (64 - len));
            h->code1[p->c] = out2;
        } else {
            h->code0[p->c] = out1;
            h->code1[p->c] = (len >= 128) ? out2 : (out2 << (128 - len));
        }
        h->cout[p->c]     = (uint8_t)len;
        h->has_code[p->c] = 1;
        return;
    }
    int index = len >> 6;
    if (index == 0) {
        out1 = out1 << 1;
        build_code(h, p->left, len + 1, out1, 0);
        out1 = out1 | 1;
        build_code(h, p->right, len + 1, out1, 0);
    } else {
        if (len % 64 != 0) out2 = out2 << 1;
        build_code(h, p->left, len + 1, out1, out2);
        out2 = out2 | 1;
        build_code(h, p->right, len + 1, out1, out2);
    }
}

/* initHuffman (src/huffman.hh:235-266): histogram, leaves inserted in symbol order, then merge
 * until one node remains.  The merge is `new_node(.., qremove(), qremove())`: GCC on x86-64
 * evaluates those two arguments right to left, so the FIRST removed node becomes the RIGHT
 * child and the second the LEFT child (pinned against the compiled reference in
 * tests/test_oracle.py). */
static int tree_init(vso_tree* h, const int32_t* s, size_t length, const uint64_t* freq_in) {
    uint64_t* freq = (uint64_t*)calloc(h->all_nodes, sizeof(uint64_t));
    if (freq_in) {
        memcpy(freq, freq_in, sizeof(uint64_t) * (h->state_num / 2));
    } else {
        for (size_t i = 0; i < length; i++) {
            uint32_t idx = (uint32_t)s[i];
            if (idx >= h->all_nodes) {
                free(freq);
                return VSO_ERR_ARG;
            }
            freq[idx]++;
        }
    }
    for (uint32_t i = 0; i < h->all_nodes; i++)
        if (freq[i]) qinsert(h, new_leaf(h, freq[i], i));
    free(freq);
    if (h->qend < 2) return VSO_ERR_ARG; /* empty input: the reference dereferences a null root */
    while (h->qend > 2) {
        int right = qremove(h);
        int left  = qremove(h);
        qinsert(h, new_internal(h, left, right));
    }
    build_code(h, h->qq[1], 0, 0, 0);
    return VSO_OK;
}

/* pad_tree_* (src/huffman.hh:374-423): preorder numbering, root 0. */
static void pad_tree(vso_tree* h, uint32_t* L, uint32_t* R, uint32_t* C, uint8_t* t, uint32_t i, int root) {
    vso_node* p = &h->pool[root];
    C[i]        = p->c;
    t[i]        = p->t;
    if (p->left >= 0) {
        h->n_inode++;
        L[i] = (uint32_t)h->n_inode;
        pad_tree(h, L, R, C, t, (uint32_t)h->n_inode, p->left);
    }
    if (p->right >= 0) {
        h->n_inode++;
        R[i] = (uint32_t)h->n_inode;
        pad_tree(h, L, R, C, t, (uint32_t)h->n_inode, p->right);
    }
}

/* Width of the serialized child indices (src/huffman.hh:425-502). */
static int tree_index_width(uint32_t node_count) { return node_count <= 256 ? 1 : (node_count <= 65536 ? 2 : 4); }

size_t vso_tree_bytes_size(uint32_t node_count) {
    int w = tree_index_width(node_count);
    return 1 + 2 * (size_t)w * node_count + 4 * (size_t)node_count + node_count;
}

static void put_index(uint8_t* dst, int w, uint32_t v) {
    if (w == 1) dst[0] = (uint8_t)v;
    else if (w == 2) {
        uint16_t x = (uint16_t)v;
        memcpy(dst, &x, 2);
    } else memcpy(dst, &v, 4);
}

static uint32_t get_index(const uint8_t* src, int w) {
    if (w == 1) return src[0];
    if (w == 2) {
        uint16_t x;
        memcpy(&x, src, 2);
        return x;
    }
    uint32_t x;
    memcpy(&x, src, 4);
    return x;
}

/* convert_HuffTree_to_bytes_anyStates (src/huffman.hh:425-502):
 * [u8 endian=0][L x n][R x n][C u32 x n][t u8 x n], host byte order (little-endian). */
static void tree_serialize(vso_tree* h, uint32_t node_count, uint8_t* out) {
    uint32_t* L = (uint32_t*)calloc(node_count, 4);
    uint32_t* R = (uint32_t*)calloc(node_count, 4);
    uint32_t* C = (uint32_t*)calloc(node_count, 4);
    uint8_t* t  = (uint8_t*)calloc(node_count, 1);
    h->n_inode  = 0;
    pad_tree(h, L, R, C, t, 0, h->qq[1]);
    int w  = tree_index_width(node_count);
    out[0] = 0;
    uint8_t* p = out + 1;
    for (uint32_t i = 0; i < node_count; i++) put_index(p + (size_t)i * w, w, L[i]);
    p += (size_t)w * node_count;
    for (uint32_t i = 0; i < node_count; i++) put_index(p + (size_t)i * w, w, R[i]);
    p += (size_t)w * node_count;
    memcpy(p, C, 4 * (size_t)node_count);
    p += 4 * (size_t)node_count;
    memcpy(p, t, node_count);
    free(L);
    free(R);
    free(C);
    free(t);
}

static void be32(uint8_t* b, uint32_t v) {
    b[0] = (uint8_t)(v >> 24);
    b[1] = (uint8_t)(v >> 16);
    b[2] = (uint8_t)(v >> 8);
    b[3] = (uint8_t)v;
}

static uint32_t rd_be32(const uint8_t* b) {
    return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}

/* Codebook of the heap-built tree for a histogram over [0, dict).  Returns node_count in
 * *node_count (2 * used symbols - 1).  lens/words may be NULL. */
int vso_huffman_codebook(const uint64_t* hist, int dict, uint8_t* lens, uint64_t* w0, uint64_t* w1,
                         uint32_t* node_count) {
    vso_tree* h = tree_create(dict * 2);
    int rc      = tree_init(h, NULL, 0, hist);
    if (rc) {
        tree_free(h);
        return rc;
    }
    uint32_t used = 0;
    for (uint32_t i = 0; i < h->state_num; i++) used += h->has_code[i];
    if (node_count) *node_count = used * 2 - 1;
    for (int i = 0; i < dict; i++) {
        if (lens) lens[i] = h->cout[i];
        if (w0) w0[i] = h->code0[i];
        if (w1) w1[i] = h->code1[i];
    }
    tree_free(h);
    return VSO_OK;
}

/* Upper bound of encode_withTree's output for n codes. */
size_t vso_huffman_bound(size_t n, int dict) {
    uint32_t nc = (uint32_t)(2 * dict);
    return 8 + vso_tree_bytes_size(nc) + n * 16 + 16;
}

/* encode_withTree (src/huffman.hh:637-662) + HuffmanEncode (:268-341).  Output:
 * [BE i32 nodeCount][BE i32 stateNum/2][tree bytes][payload].  The payload is the MSB-first
 * concatenation of the codewords, ceil(bits/8) bytes, last byte zero-padded. */
int vso_huffman_encode(const int32_t* s, size_t n, int dict, uint8_t* out, size_t cap, size_t* out_size) {
    vso_tree* h = tree_create(dict * 2);
    int rc      = tree_init(h, s, n, NULL);
    if (rc) {
        tree_free(h);
        return rc;
    }
    uint32_t used = 0;
    for (uint32_t i = 0; i < h->state_num; i++) used += h->has_code[i];
    uint32_t node_count = used * 2 - 1;
    size_t tsz          = vso_tree_bytes_size(node_count);
    if (8 + tsz > cap) {
        tree_free(h);
        return VSO_ERR_CAPACITY;
    }
    be32(out, node_count);
    be32(out + 4, h->state_num / 2);
    tree_serialize(h, node_count, out + 8);
    uint8_t* pay = out + 8 + tsz;
    size_t pcap  = cap - 8 - tsz;
    /* MSB-first bit writer with a 64-bit accumulator (same bytes as HuffmanEncode's byte loop) */
    uint64_t bit = 0, acc = 0;
    int nacc     = 0; /* bits pending in acc (left-aligned) */
    size_t wpos  = 0;
    for (size_t i = 0; i < n; i++) {
        uint32_t sym = (uint32_t)s[i];
        int len      = h->cout[sym];
        for (int part = 0; part < 2 && len > 0; part++) {
            int take      = len > 64 ? 64 : len;
            uint64_t word = part == 0 ? h->code0[sym] : h->code1[sym];
            /* left-aligned `take` bits of word */
            while (take > 0) {
                int room = 64 - nacc;
                int t    = take < room ? take : room;
                uint64_t bits = word >> (64 - t);
                acc |= (t == 64) ? bits : (bits << (64 - nacc - t));
                nacc += t;
                word = (t == 64) ? 0 : (word << t);
                take -= t;
                bit += (uint64_t)t;
                while (nacc >= 8) {
                    if (wpos >= pcap) {
                        tree_free(h);
                        return VSO_ERR_CAPACITY;
                    }
                    pay[wpos++] = (uint8_t)(acc >> 56);
                    acc <<= 8;
                    nacc -= 8;
                }
            }
            len -= 64;
        }
    }
    if (nacc > 0) {
        if (wpos >= pcap) {
            tree_free(h);
            return VSO_ERR_CAPACITY;
        }
        pay[wpos++] = (uint8_t)(acc >> 56);
    }
    *out_size = 8 + tsz + (size_t)((bit + 7) >> 3);
    tree_free(h);
    return VSO_OK;
}

/* decode_withTree (src/huffman.hh:679-691) + reconstruct_HuffTree_from_bytes_anyStates (:561-635)
 * + decode (:343-372).  Walks the serialized tree directly: child index 0 means "no child".
 * Bounded: a stream that ends before n symbols or a malformed tree returns VSO_ERR_CORRUPT. */
int vso_huffman_decode(const uint8_t* in, size_t in_len, size_t n, int32_t* out) {
    if (in_len < 8) return VSO_ERR_CORRUPT;
    uint32_t nc = rd_be32(in);
    if (nc == 0) return VSO_ERR_CORRUPT;
    size_t tsz = vso_tree_bytes_size(nc);
    if (8 + tsz > in_len) return VSO_ERR_CORRUPT;
    int w              = tree_index_width(nc);
    const uint8_t* tb  = in + 8 + 1;
    const uint8_t* Lb  = tb;
    const uint8_t* Rb  = tb + (size_t)w * nc;
    const uint8_t* Cb  = tb + 2 * (size_t)w * nc;
    const uint8_t* Tb  = Cb + 4 * (size_t)nc;
    const uint8_t* pay = in + 8 + tsz;
    size_t pbits       = (in_len - 8 - tsz) * 8;
    /* The reference builds the root from (C[0], t[0]) only when nodeCount <= 256 and as an
     * internal node otherwise (src/huffman.hh:577,602,627). */
    int root_leaf = (nc <= 256) ? Tb[0] : 0;
    if (root_leaf) {
        uint32_t c;
        memcpy(&c, Cb, 4);
        for (size_t k = 0; k < n; k++) out[k] = (int32_t)c;
        return VSO_OK;
    }
    uint32_t* ch = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)nc);
    int32_t* leaf = (int32_t*)malloc(sizeof(int32_t) * (size_t)nc);
    if (!ch || !leaf) {
        free(ch);
        free(leaf);
        return VSO_ERR_ARG;
    }
    for (uint32_t k = 0; k < nc; k++) {
        ch[2 * k]     = get_index(Lb + (size_t)k * w, w);
        ch[2 * k + 1] = get_index(Rb + (size_t)k * w, w);
        uint32_t c;
        memcpy(&c, Cb + 4 * (size_t)k, 4);
        leaf[k] = (k != 0 && Tb[k]) ? (int32_t)c : -1;
    }
    uint32_t node = 0;
    size_t count = 0, i = 0;
    int rc = VSO_OK;
    while (count < n) {
        if (i >= pbits) {
            rc = VSO_ERR_CORRUPT;
            break;
        }
        int bitv      = (pay[i >> 3] >> (7 - (i & 7))) & 1;
        uint32_t next = ch[2 * node + (uint32_t)bitv];
        if (next == 0 || next >= nc) {
            rc = VSO_ERR_CORRUPT;
            break;
        }
        node = next;
        i++;
        if (leaf[node] >= 0) {
            out[count++] = leaf[node];
            node         = 0;
        }
    }
    free(ch);
    free(leaf);
    return rc;
}

/* ------------------------------------------------------------------------------------------ */
/* Whole-field compress / decompress (src/vecsz_interface.hh:31-229, 232-375), with optional    */
/* padding, without the lossless pass.  The packed block (src/utils/datapack.hh:17-29):         */
/*   i32 ndim; i32 dims[ndim]; f64 eb (the user's eb); u64 {n_pad, huff_bytes, n_outliers};     */
/*   f32 pad[n_pad]; huffman bytes; f32 outliers[n_outliers]                                     */
/* ------------------------------------------------------------------------------------------ */

size_t vso_compress_bound(int ndim, size_t n, int dict) {
    return 4 * (size_t)(ndim + 1) + 8 + 24 + vso_huffman_bound(n, dict) + 4 * n;
}

/* ... plus the pad section of -p (vso_pad_count floats). */
size_t vso_compress_bound_pad(int ndim, const size_t* dims, int bs, int dict, int pad_mode) {
    size_t d0 = dims[0], d1 = ndim > 1 ? dims[1] : 1, d2 = ndim > 2 ? dims[2] : 1;
    return vso_compress_bound(ndim, d0 * d1 * d2, dict) + 4 * vso_pad_count(ndim, d0, d1, d2, bs, pad_mode);
}

/* timings (optional, seconds): [0] value range, [1] dual-quant, [2] Huffman, [3] outlier gather.
 * pad_mode / pad_type / pad_const: -p (VSO_PAD_*, VSO_PADV_*); the pad values follow the header
 * (src/utils/datapack.hh:23). */
int vso_compress_pad(const float* x, int ndim, const size_t* dims, int bs, int dict, double eb, int r2r, int pad_mode,
                     int pad_type, float pad_const, uint8_t* out, size_t cap, size_t* out_size, size_t* n_outlier,
                     double* eb_final_out, double* timings) {
    if (ndim < 1 || ndim > 3 || dict < 2 || dict > 65536 || eb <= 0) return VSO_ERR_ARG;
    size_t d0 = dims[0], d1 = ndim > 1 ? dims[1] : 1, d2 = ndim > 2 ? dims[2] : 1;
    size_t n  = d0 * d1 * d2;
    if (n == 0) return VSO_ERR_ARG;
    double t0 = now_s();
    double ebf = eb;
    if (r2r) {
        double range = vso_value_range(x, n);
        if (range == 0) return VSO_ERR_ARG; /* the reference exits: src/types.cc:51-54 */
        ebf *= range;
    }
    double ebs[4];
    vso_eb_family(ebf, ebs);
    double t1       = now_s();
    int32_t* code   = (int32_t*)calloc(n, sizeof(int32_t));
    float* outl     = (float*)calloc(n, sizeof(float));
    size_t npad     = vso_pad_count(ndim, d0, d1, d2, bs, pad_mode);
    float* pads     = (float*)calloc(npad ? npad : 1, sizeof(float));
    int rc = vso_dualquant_pad(x, ndim, d0, d1, d2, bs, dict / 2, ebs[3], pad_mode, pad_type, pad_const, code, outl,
                               pads);
    size_t hdr = 4 * (size_t)(ndim + 1) + 8 + 24 + 4 * npad;
    if (!rc && hdr > cap) rc = VSO_ERR_CAPACITY;
    if (rc) {
        free(code);
        free(outl);
        free(pads);
        return rc;
    }
    memcpy(out + hdr - 4 * npad, pads, 4 * npad);
    free(pads);
    double t2 = now_s();
    size_t hsz = 0;
    rc         = vso_huffman_encode(code, n, dict, out + hdr, cap > hdr ? cap - hdr : 0, &hsz);
    if (rc) {
        free(code);
        free(outl);
        return rc;
    }
    double t3 = now_s();
    size_t pos = hdr + hsz;
    size_t k   = 0;
    for (size_t i = 0; i < n; i++)
        if (code[i] == 0) {
            if (pos + 4 * (k + 1) > cap) {
                free(code);
                free(outl);
                return VSO_ERR_CAPACITY;
            }
            memcpy(out + pos + 4 * k, &outl[i], 4);
            k++;
        }
    double t4 = now_s();
    int32_t meta[4] = {ndim, (int32_t)d0, (int32_t)d1, (int32_t)d2};
    memcpy(out, meta, 4 * (size_t)(ndim + 1));
    memcpy(out + 4 * (ndim + 1), &eb, 8);
    uint64_t lens[3] = {(uint64_t)npad, (uint64_t)hsz, (uint64_t)k};
    memcpy(out + 4 * (ndim + 1) + 8, lens, 24);
    *out_size = pos + 4 * k;
    if (n_outlier) *n_outlier = k;
    if (eb_final_out) *eb_final_out = ebf;
    if (timings) {
        timings[0] = t1 - t0;
        timings[1] = t2 - t1;
        timings[2] = t3 - t2;
        timings[3] = t4 - t3;
    }
    free(code);
    free(outl);
    return VSO_OK;
}

int vso_compress(const float* x, int ndim, const size_t* dims, int bs, int dict, double eb, int r2r, uint8_t* out,
                 size_t cap, size_t* out_size, size_t* n_outlier, double* eb_final_out, double* timings) {
    return vso_compress_pad(x, ndim, dims, bs, dict, eb, r2r, VSO_PAD_NONE, VSO_PADV_CONST, 0.0f, out, cap, out_size,
                            n_outlier, eb_final_out, timings);
}

/* Parse the packed block's header.  dims_out[3] (missing dims = 1). */
int vso_parse_header(const uint8_t* in, size_t len, int* ndim, size_t* dims_out, double* eb, uint64_t* lens) {
    if (len < 4) return VSO_ERR_CORRUPT;
    int32_t nd;
    memcpy(&nd, in, 4);
    if (nd < 1 || nd > 3) return VSO_ERR_CORRUPT;
    size_t hdr = 4 * (size_t)(nd + 1) + 8 + 24;
    if (len < hdr) return VSO_ERR_CORRUPT;
    int32_t d[3] = {1, 1, 1};
    memcpy(d, in + 4, 4 * (size_t)nd);
    for (int i = 0; i < 3; i++) {
        if (d[i] <= 0) return VSO_ERR_CORRUPT;
        dims_out[i] = (size_t)d[i];
    }
    memcpy(eb, in + 4 * (nd + 1), 8);
    memcpy(lens, in + 4 * (nd + 1) + 8, 24);
    *ndim = nd;
    if (hdr + 4 * lens[0] + lens[1] + 4 * lens[2] > len) return VSO_ERR_CORRUPT;
    return VSO_OK;
}

/* Decompress a packed block.  value_range > 0 selects r2r (eb_final = eb * value_range), which the
 * reference gets by re-reading the original field (src/vecsz_interface.hh:280-284).
 * timings (optional): [0] Huffman decode, [1] outlier scatter, [2] reverse dual-quant. */
int vso_decompress(const uint8_t* in, size_t len, int bs, int dict, double value_range, float* xhat, size_t n_cap,
                   double* timings) {
    int ndim;
    size_t dims[3];
    double eb;
    uint64_t lens[3];
    int rc = vso_parse_header(in, len, &ndim, dims, &eb, lens);
    if (rc) return rc;
    size_t n = dims[0] * dims[1] * dims[2];
    if (n > n_cap) return VSO_ERR_CAPACITY;
    double ebf = eb;
    if (value_range > 0) ebf *= value_range;
    double ebs[4];
    vso_eb_family(ebf, ebs);
    size_t hdr         = 4 * (size_t)(ndim + 1) + 8 + 24;
    const uint8_t* hp  = in + hdr + 4 * lens[0];
    const float* outs  = (const float*)(const void*)(hp + lens[1]);
    int32_t* code      = (int32_t*)malloc(n * sizeof(int32_t));
    float* dense       = (float*)malloc(n * sizeof(float));
    float* outl_copy   = (float*)malloc((lens[2] ? lens[2] : 1) * sizeof(float));
    float* pads        = (float*)malloc((lens[0] ? lens[0] : 1) * sizeof(float));
    memcpy(outl_copy, outs, lens[2] * sizeof(float));
    memcpy(pads, in + hdr, lens[0] * sizeof(float));
    double t0 = now_s();
    rc        = vso_huffman_decode(hp, lens[1], n, code);
    if (rc) {
        free(code);
        free(dense);
        free(outl_copy);
        free(pads);
        return rc;
    }
    double t1 = now_s();
    size_t zeros = 0;
    for (size_t i = 0; i < n; i++) zeros += code[i] == 0;
    if (zeros > lens[2]) {
        free(code);
        free(dense);
        free(outl_copy);
        free(pads);
        return VSO_ERR_CORRUPT;
    }
    vso_scatter_outliers(code, outl_copy, n, dense);
    double t2 = now_s();
    rc = vso_xlorenzo_pad(code, dense, ndim, dims[0], dims[1], dims[2], bs, dict / 2, ebs[2], pads, lens[0], xhat);
    double t3 = now_s();
    if (timings) {
        timings[0] = t1 - t0;
        timings[1] = t2 - t1;
        timings[2] = t3 - t2;
    }
    free(code);
    free(dense);
    free(outl_copy);
    free(pads);
    return rc;
}

int vso_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
