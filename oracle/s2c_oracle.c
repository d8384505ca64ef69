/*
 * CPU oracle for the strands-to-cards raster path -- TEST INFRASTRUCTURE ONLY
 * (checker for tests/, __graft_entry__.smoke() and the CPU baseline of bench.py).
 *
 * Each function cites the reference kernel it restates (paths inside the reference
 * project).  Build: oracle/Makefile (-O2 -ffp-contract=off, OpenMP).  See s2c_oracle.h
 * for the FP32 bit-mirror / FP64 split and the arithmetic-model flags.
 */
#include "s2c_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* the model pinned against the reference's outputs (tests/golden) */
#define OR_DEFAULT_MODEL (OR_FMA_DDA_SPAN | OR_FMA_DDA_PERSP | OR_FMA_TRI_RECT | OR_FMA_TRI_Q | \
                          OR_FMA_TRI_A | OR_FMA_AA)

static int g_model = OR_DEFAULT_MODEL;
static int g_dz = 2, g_tz = 2, g_tw = 1;  /* contraction shapes of the dot products */
void or_set_zvariant(int dda, int tri_z, int tri_w) { g_dz = dda; g_tz = tri_z; g_tw = tri_w; }

/* three-term dot product ((a0 b0 + a1 b1) + a2 b2) under contraction shape v */
static inline float dot3(int v, float a0, float b0, float a1, float b1, float a2, float b2) {
    switch (v) {
    case 0: return a0 * b0 + a1 * b1 + a2 * b2;
    case 1: return fmaf(a2, b2, fmaf(a0, b0, a1 * b1));
    case 2: return fmaf(a2, b2, fmaf(a1, b1, a0 * b0));
    case 3: return fmaf(a2, b2, a0 * b0 + a1 * b1);
    case 4: return fmaf(a0, b0, a1 * b1) + a2 * b2;
    case 5: return fmaf(a0, b0, fmaf(a1, b1, a2 * b2));
    case 6: return fmaf(a1, b1, fmaf(a0, b0, a2 * b2));
    case 7: return fmaf(a1, b1, a0 * b0) + a2 * b2;
    default: return fmaf(a0, b0, fmaf(a2, b2, a1 * b1));
    }
}
static int g_threads = 0;
#define HAS(f) ((g_model & (f)) != 0)

int or_version(void) { return 1; }
void or_set_model(int flags) { g_model = flags < 0 ? OR_DEFAULT_MODEL : flags; }
int or_get_model(void) { return g_model; }
void or_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

/* float -> int with the saturating, NaN -> 0 semantics of cvt.rzi.s32.f32 */
static inline int f2i(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}
static inline float fmax_macro(float a, float b) { return a > b ? a : b; } /* cuda_common.cuh MAX */
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int wrap_sub(int a, int b) { return (int)(int32_t)((uint32_t)a - (uint32_t)b); }

/* ================================================================================== */
/* DDA (dda.cu)                                                                        */
/* ================================================================================== */

/* dda.cu:9-87 (dda_compute_span_kernel) for one primitive */
static int32_t span_one(int32_t eid, int H, int W, int V, const float* pos, int E,
                        const int32_t* edges, float* sl, float* sp) {
    const int b = eid / E, e = eid % E;
    const int v0 = edges[2 * (int64_t)e], v1 = edges[2 * (int64_t)e + 1];
    const float* pp = pos + (int64_t)b * V * 4;
    const float x0n = pp[v0 * 4 + 0] / pp[v0 * 4 + 3];
    const float y0n = pp[v0 * 4 + 1] / pp[v0 * 4 + 3];
    const float x1n = pp[v1 * 4 + 0] / pp[v1 * 4 + 3];
    const float y1n = pp[v1 * 4 + 1] / pp[v1 * 4 + 3];
    const float fH = (float)H, fW = (float)W;
    float x0 = 0.5f * (x0n + 1.f) * fW;
    float y0 = 0.5f * (1.f - y0n) * fH;
    float x1 = 0.5f * (x1n + 1.f) * fW;
    float y1 = 0.5f * (1.f - y1n) * fH;
    const float dx = x1 - x0, dy = y1 - y0;
    sl[0] = sl[1] = 0.f;
    sp[0] = sp[1] = sp[2] = sp[3] = 0.f;
    if (dx == 0.f && dy == 0.f) return 0;
    if (fabsf(dx) >= fabsf(dy)) {
        const float s = dy / dx;
        sl[0] = 0.f; sl[1] = s;
        if (x0 > x1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
        const float fsx = fmax_macro(floorf(x0), 0.f);
        const float fsy = HAS(OR_FMA_DDA_SPAN) ? fmaf(s, fsx - x0, y0) : y0 + s * (fsx - x0);
        const int xs = f2i(fsx);
        const int xe = imin(f2i(floorf(x1)), W - 1) + 1;
        sp[0] = fsx; sp[1] = fsy; sp[2] = x0 - fsx; sp[3] = x1 - fsx;
        return imax(wrap_sub(xe, xs), 0);
    } else {
        const float s = dx / dy;
        sl[0] = 1.f; sl[1] = s;
        if (y0 > y1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
        const float fsy = fmax_macro(floorf(y0), 0.f);
        const float fsx = HAS(OR_FMA_DDA_SPAN) ? fmaf(s, fsy - y0, x0) : x0 + s * (fsy - y0);
        const int ys = f2i(fsy);
        const int ye = imin(f2i(floorf(y1)), H - 1) + 1;
        sp[0] = fsx; sp[1] = fsy; sp[2] = y0 - fsy; sp[3] = y1 - fsy;
        return imax(wrap_sub(ye, ys), 0);
    }
}

void or_dda_span(int64_t P, const int32_t* edge_ids, int H, int W, int V, const float* pos,
                 int E, const int32_t* edges, int32_t* counts, float* slopes, float* spans) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < P; ++p)
        counts[p] = span_one(edge_ids ? edge_ids[p] : (int32_t)p, H, W, V, pos, E, edges,
                             slopes + 2 * p, spans + 4 * p);
}

/* dda.cu:124-144 (perspective_correct_interpolate) */
static inline float persp_t1(int H, int W, const float* p0, const float* p1, float x, float y,
                             float axis) {
    float t0, t1;
    if (axis == 0.f) {
        const float qx = -1.f + 2.f * (x / (float)W);
        const float a = HAS(OR_FMA_DDA_PERSP) ? fmaf(-qx, p0[3], p0[0]) : p0[0] - qx * p0[3];
        const float b = HAS(OR_FMA_DDA_PERSP) ? fmaf(-qx, p1[3], p1[0]) : p1[0] - qx * p1[3];
        t0 = fabsf(b);
        t1 = fabsf(a);
    } else {
        const float qy = -1.f + 2.f * (y / (float)H);
        const float a = HAS(OR_FMA_DDA_PERSP) ? fmaf(-qy, p0[3], -p0[1]) : -p0[1] - qy * p0[3];
        const float b = HAS(OR_FMA_DDA_PERSP) ? fmaf(-qy, p1[3], -p1[1]) : -p1[1] - qy * p1[3];
        t0 = fabsf(b);
        t1 = fabsf(a);
    }
    const float den = t0 + t1;
    if (den < 1e-6f) return 0.5f;
    return t1 / den;
}

static inline float lerp2(float t0, float a, float t1, float b) {
    switch (g_dz) {
    case 0: return t0 * a + t1 * b;
    case 1: return fmaf(t0, a, t1 * b);
    default: return fmaf(t1, b, t0 * a);
    }
}

/* dda.cu:146-225 (dda_compute_fragments_kernel) for fragment k of primitive p.
 * Returns 1 and fills (b,h,w)/(axis,t1,z,e+1) when the fragment survives. */
static inline int frag_one(int32_t eid, int k, const float* sl, const float* sp, int H, int W,
                           int V, const float* pos, int E, const int32_t* edges,
                           int32_t* pix, float* at) {
    const int b = eid / E, e = eid % E;
    const float d = fminf(fmaxf((float)k + 0.5f, sp[2]), sp[3]);
    const float axis = sl[0], s = sl[1];
    float x, y;
    if (axis == 0.f) {
        x = sp[0] + d;
        y = HAS(OR_FMA_DDA_STEP) ? fmaf(d, s, sp[1]) : sp[1] + d * s;
    } else {
        x = HAS(OR_FMA_DDA_STEP) ? fmaf(d, s, sp[0]) : sp[0] + d * s;
        y = sp[1] + d;
    }
    const int h = f2i(floorf(y)), w = f2i(floorf(x));
    if (h < 0 || h >= H || w < 0 || w >= W) return 0;
    const int v0 = edges[2 * (int64_t)e], v1 = edges[2 * (int64_t)e + 1];
    const float* pp = pos + (int64_t)b * V * 4;
    const float* p0 = pp + (int64_t)v0 * 4;
    const float* p1 = pp + (int64_t)v1 * 4;
    const float t1 = persp_t1(H, W, p0, p1, x, y, axis);
    const float t0 = 1.f - t1;
    const float pz = lerp2(t0, p0[2], t1, p1[2]);
    const float pw = lerp2(t0, p0[3], t1, p1[3]);
    const float zw = pz / pw;
    if (!isfinite(zw) || zw < -1.f || zw > 1.f) return 0;
    pix[0] = b; pix[1] = h; pix[2] = w;
    at[0] = axis; at[1] = t1; at[2] = zw; at[3] = (float)(e + 1);
    return 1;
}

void or_dda_fragments(int64_t P, const int32_t* prefix, const int32_t* edge_ids,
                      const float* slopes, const float* spans, int H, int W, int V,
                      const float* pos, int E, const int32_t* edges,
                      int32_t* frag_pix, float* frag_attrs) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t p = 0; p < P; ++p) {
        const int64_t base = p ? prefix[p - 1] : 0;
        const int64_t cnt = prefix[p] - base;
        const int32_t eid = edge_ids ? edge_ids[p] : (int32_t)p;
        for (int64_t k = 0; k < cnt; ++k) {
            int32_t* px = frag_pix + 3 * (base + k);
            px[0] = px[1] = px[2] = -1;
            frag_one(eid, (int)k, slopes + 2 * p, spans + 4 * p, H, W, V, pos, E, edges, px,
                     frag_attrs + 4 * (base + k));
        }
    }
}

/* dda_compute_fragments followed by cluster_mask_from_fragments (rasterize.cu:474-498):
 * the fragment's prim id travels as float(e+1) in the reference, so it is rounded the
 * same way here. */
void or_dda_cluster_bitset(int B, int H, int W, int V, const float* pos, int E,
                           const int32_t* edges, const int32_t* edge_ids, int64_t P,
                           const int32_t* prim2cluster, int S, int32_t* bitset) {
    const int64_t words = (int64_t)B * H * W * S;
    memset(bitset, 0, (size_t)words * sizeof(int32_t));
    if (!edge_ids) P = (int64_t)B * E;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t p = 0; p < P; ++p) {
        float sl[2], sp[4];
        const int32_t eid = edge_ids ? edge_ids[p] : (int32_t)p;
        const int cnt = span_one(eid, H, W, V, pos, E, edges, sl, sp);
        for (int k = 0; k < cnt; ++k) {
            int32_t px[3];
            float at[4];
            if (!frag_one(eid, k, sl, sp, H, W, V, pos, E, edges, px, at)) continue;
            const int prim = f2i(at[3]) - 1;
            if (prim < 0) continue;
            const int c = prim2cluster[prim];
            const int64_t word = (((int64_t)px[0] * H + px[1]) * W + px[2]) * S + c / 32;
            __atomic_fetch_or(&bitset[word], (int32_t)(1u << (c % 32)), __ATOMIC_RELAXED);
        }
    }
}

/* ================================================================================== */
/* triangles (rasterize.cu)                                                            */
/* ================================================================================== */

/* rasterize.cu:9-59 */
void or_tri_rects(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                  int32_t* rects, int32_t* counts) {
    const float fH = (float)H, fW = (float)W;
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < (int64_t)B * T; ++idx) {
        const int64_t b = idx / T, t = idx % T;
        float x0 = fW, y0 = fH, x1 = 0.f, y1 = 0.f;
        for (int i = 0; i < 3; ++i) {
            const float* p = pos + (b * V + tri[t * 3 + i]) * 4;
            const float inv_w = 1.f / p[3];
            const float ax = HAS(OR_FMA_TRI_RECT) ? fmaf(p[0], inv_w, 1.f) : 1.f + p[0] * inv_w;
            const float ay = HAS(OR_FMA_TRI_RECT) ? fmaf(-p[1], inv_w, 1.f) : 1.f - p[1] * inv_w;
            const float x = 0.5f * ax * fW;
            const float y = 0.5f * ay * fH;
            x0 = isnan(x) ? x0 : fminf(x, x0);
            x1 = isnan(x) ? x1 : fmaxf(x, x1);
            y0 = isnan(y) ? y0 : fminf(y, y0);
            y1 = isnan(y) ? y1 : fmaxf(y, y1);
        }
        const int h0 = imax(f2i(floorf(y0)), 0);
        const int h1 = imin(f2i(floorf(y1)), H - 1) + 1;
        const int w0 = imax(f2i(floorf(x0)), 0);
        const int w1 = imin(f2i(floorf(x1)), W - 1) + 1;
        const int hl = imax(wrap_sub(h1, h0), 0), wl = imax(wrap_sub(w1, w0), 0);
        rects[idx * 4 + 0] = h0; rects[idx * 4 + 1] = hl;
        rects[idx * 4 + 2] = w0; rects[idx * 4 + 3] = wl;
        counts[idx] = (int32_t)((uint32_t)hl * (uint32_t)wl);
    }
}

static inline float cross2(float a, float b, float c, float d) {
    if (HAS(OR_FMA_TRI_A)) return fmaf(a, b, -(c * d));
    if (HAS(OR_FMA_TRI_A_ALT)) return fmaf(-c, d, a * b);
    return a * b - c * d;
}

/* rasterize.cu:90-172 for one (b, t) and pixel (x, y); returns 1 when covered */
static inline int tri_cover(int H, int W, const float* P0, const float* P1, const float* P2,
                            int x, int y, float* b0o, float* b1o, float* zo) {
    const float px = -1.f + 2.f * ((float)x + 0.5f) / (float)W;
    const float py = -1.f + 2.f * ((float)y + 0.5f) / (float)H;
    const int fq = HAS(OR_FMA_TRI_Q);
    const float q0x = fq ? fmaf(-px, P0[3], P0[0]) : P0[0] - px * P0[3];
    const float q0y = fq ? fmaf(-py, P0[3], -P0[1]) : -P0[1] - py * P0[3];
    const float q1x = fq ? fmaf(-px, P1[3], P1[0]) : P1[0] - px * P1[3];
    const float q1y = fq ? fmaf(-py, P1[3], -P1[1]) : -P1[1] - py * P1[3];
    const float q2x = fq ? fmaf(-px, P2[3], P2[0]) : P2[0] - px * P2[3];
    const float q2y = fq ? fmaf(-py, P2[3], -P2[1]) : -P2[1] - py * P2[3];
    const float A0 = cross2(q1x, q2y, q1y, q2x);
    const float A1 = cross2(q2x, q0y, q2y, q0x);
    const float A2 = cross2(q0x, q1y, q0y, q1x);
    const float A = A0 + A1 + A2;
    if (A == 0.f) return 0;
    const float invA = 1.f / A;
    const float b0 = A0 * invA, b1 = A1 * invA;
    float zc, wc;
    zc = dot3(g_tz, A0, P0[2], A1, P1[2], A2, P2[2]);
    wc = dot3(g_tw, A0, P0[3], A1, P1[3], A2, P2[3]);
    const float z = zc / wc;
    if (!isfinite(b0) || !isfinite(b1) || !isfinite(z)) return 0;
    if (b0 < 0.f || b1 < 0.f || b0 + b1 > 1.f || z < -1.f || z > 1.f) return 0;
    *b0o = b0; *b1o = b1; *zo = z;
    return 1;
}

void or_tri_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                      const int32_t* rects, const int32_t* prefix,
                      int32_t* frag_pix, float* frag_attrs) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t idx = 0; idx < (int64_t)B * T; ++idx) {
        const int64_t base = idx ? prefix[idx - 1] : 0;
        const int64_t cnt = prefix[idx] - base;
        const int b = (int)(idx / T), t = (int)(idx % T);
        const int h0 = rects[idx * 4 + 0], hl = rects[idx * 4 + 1];
        const int w0 = rects[idx * 4 + 2], wl = rects[idx * 4 + 3];
        const float* pb = pos + (int64_t)b * V * 4;
        const float* P0 = pb + (int64_t)tri[t * 3 + 0] * 4;
        const float* P1 = pb + (int64_t)tri[t * 3 + 1] * 4;
        const float* P2 = pb + (int64_t)tri[t * 3 + 2] * 4;
        for (int64_t k = 0; k < cnt; ++k) {
            int32_t* px = frag_pix + 3 * (base + k);
            px[0] = px[1] = px[2] = -1;
            if (wl <= 0 || hl <= 0) continue;
            const int y = h0 + (int)(k / wl), x = w0 + (int)(k % wl);
            if (x < 0 || x >= W || y < 0 || y >= H) continue;
            float b0, b1, z;
            if (!tri_cover(H, W, P0, P1, P2, x, y, &b0, &b1, &z)) continue;
            float* at = frag_attrs + 4 * (base + k);
            px[0] = b; px[1] = y; px[2] = x;
            at[0] = b0; at[1] = b1; at[2] = z; at[3] = (float)(t + 1);
        }
    }
}

/* rasterize.cu:336-365, but order-preserving */
int64_t or_filter_valid(int64_t F, const int32_t* pix, const float* attrs, int32_t* pix_out,
                        float* attrs_out) {
    int64_t n = 0;
    for (int64_t i = 0; i < F; ++i) {
        if (pix[3 * i] < 0) continue;
        memcpy(pix_out + 3 * n, pix + 3 * i, 3 * sizeof(int32_t));
        memcpy(attrs_out + 4 * n, attrs + 4 * i, 4 * sizeof(float));
        ++n;
    }
    return n;
}

/* rasterize.cu:198-278: key = (bits(z + 2) << 32) | fragment index, minimum wins */
void or_depth_test(int B, int H, int W, int64_t F, const int32_t* frag_pix,
                   const float* frag_attrs, float* rast) {
    const int64_t npix = (int64_t)B * H * W;
    int64_t* key = (int64_t*)malloc((size_t)npix * sizeof(int64_t));
    for (int64_t i = 0; i < npix; ++i) key[i] = INT64_MAX;
    for (int64_t i = 0; i < F; ++i) {
        const int64_t pix = ((int64_t)frag_pix[3 * i] * H + frag_pix[3 * i + 1]) * W + frag_pix[3 * i + 2];
        const float zz = frag_attrs[4 * i + 2] + 2.f;
        int32_t zb;
        memcpy(&zb, &zz, 4);
        const int64_t k = (int64_t)(((uint64_t)(int64_t)zb << 32) | (uint32_t)i);
        if (k < key[pix]) key[pix] = k;
    }
    memset(rast, 0, (size_t)npix * 4 * sizeof(float));
    for (int64_t p = 0; p < npix; ++p) {
        if (key[p] == INT64_MAX) continue;
        const int32_t fi = (int32_t)(key[p] & 0xFFFFFFFFLL);
        if (fi < 0) continue;
        memcpy(rast + 4 * p, frag_attrs + 4 * (int64_t)fi, 4 * sizeof(float));
    }
    free(key);
}

/* rasterize.cu:474-498 */
void or_cluster_mask(int64_t F, const int32_t* frag_pix, const float* frag_attrs,
                     const int32_t* prim2cluster, int H, int W, int S, int32_t* bitset) {
    for (int64_t i = 0; i < F; ++i) {
        const int prim = f2i(frag_attrs[4 * i + 3]) - 1;
        if (prim < 0) continue;
        const int c = prim2cluster[prim];
        const int64_t word = (((int64_t)frag_pix[3 * i] * H + frag_pix[3 * i + 1]) * W + frag_pix[3 * i + 2]) * S + c / 32;
        bitset[word] |= (int32_t)(1u << (c % 32));
    }
}

/* rasterize.cu:367-438, evaluated in FP64 */
void or_interpolate(int B, int H, int W, const float* rast, int C, const float* attr,
                    const int32_t* tri, double* image) {
    const int64_t npix = (int64_t)B * H * W;
    for (int64_t p = 0; p < npix; ++p) {
        const double b0 = rast[4 * p], b1 = rast[4 * p + 1], b2 = 1.0 - b0 - b1;
        const int t = f2i(rast[4 * p + 3]) - 1;
        for (int c = 0; c < C; ++c) image[p * C + c] = 0.0;
        if (t < 0) continue;
        const float* a0 = attr + (int64_t)C * tri[3 * t];
        const float* a1 = attr + (int64_t)C * tri[3 * t + 1];
        const float* a2 = attr + (int64_t)C * tri[3 * t + 2];
        for (int c = 0; c < C; ++c) image[p * C + c] = b0 * a0[c] + b1 * a1[c] + b2 * a2[c];
    }
}

void or_interpolate_backward(int B, int H, int W, const float* rast, int C,
                             const float* d_image, const int32_t* tri, double* d_attr) {
    const int64_t npix = (int64_t)B * H * W;
    for (int64_t p = 0; p < npix; ++p) {
        const double b0 = rast[4 * p], b1 = rast[4 * p + 1], b2 = 1.0 - b0 - b1;
        const int t = f2i(rast[4 * p + 3]) - 1;
        if (t < 0) continue;
        for (int c = 0; c < C; ++c) {
            const double g = d_image[p * C + c];
            d_attr[(int64_t)C * tri[3 * t] + c] += g * b0;
            d_attr[(int64_t)C * tri[3 * t + 1] + c] += g * b1;
            d_attr[(int64_t)C * tri[3 * t + 2] + c] += g * b2;
        }
    }
}

/* dda.cu:258-327, evaluated in FP64 */
void or_dda_interpolate(int B, int H, int W, const float* rast, int C, const float* attr,
                        const int32_t* edges, double* image) {
    const int64_t npix = (int64_t)B * H * W;
    for (int64_t p = 0; p < npix; ++p) {
        const double t1 = rast[4 * p + 1], t0 = 1.0 - t1;
        const int e = f2i(rast[4 * p + 3]) - 1;
        for (int c = 0; c < C; ++c) image[p * C + c] = 0.0;
        if (e < 0) continue;
        const float* a0 = attr + (int64_t)C * edges[2 * e];
        const float* a1 = attr + (int64_t)C * edges[2 * e + 1];
        for (int c = 0; c < C; ++c) image[p * C + c] = t0 * a0[c] + t1 * a1[c];
    }
}

void or_dda_interpolate_backward(int B, int H, int W, const float* rast, int C,
                                 const float* d_image, const int32_t* edges, double* d_attr) {
    const int64_t npix = (int64_t)B * H * W;
    for (int64_t p = 0; p < npix; ++p) {
        const double t1 = rast[4 * p + 1], t0 = 1.0 - t1;
        const int e = f2i(rast[4 * p + 3]) - 1;
        if (e < 0) continue;
        for (int c = 0; c < C; ++c) {
            const double g = d_image[p * C + c];
            d_attr[(int64_t)C * edges[2 * e] + c] += g * t0;
            d_attr[(int64_t)C * edges[2 * e + 1] + c] += g * t1;
        }
    }
}

/* ================================================================================== */
/* antialias (antialias.cu, compact_utils.cu)                                          */
/* ================================================================================== */


static inline int third_vertex(const int32_t* tri, int t, int v0, int v1) {
    /* antialias.cu:7-15 */
    const int i0 = tri[t * 3], i1 = tri[t * 3 + 1], i2 = tri[t * 3 + 2];
    return (i0 != v0 && i0 != v1) ? i0 : (i1 != v0 && i1 != v1) ? i1 : (i2 != v0 && i2 != v1) ? i2 : -1;
}

static int g_aa = 1;
void or_set_aavariant(int v) { g_aa = v; }
static inline float dot2(float a, float b, float c, float d) {
    if (!HAS(OR_FMA_AA)) return a * b + c * d;
    return g_aa == 1 ? fmaf(a, b, c * d) : fmaf(c, d, a * b);
}

/* antialias.cu:38-94.  nvcc fuses the projection multiply of the second operand into
 * each coordinate difference (x1 - x0 -> fma(W/2, 1 + ndc_x1, -x0)), so the differences
 * are restated that way; the first vertex's pixel coordinates are rounded. */
static inline void proj_a(const float* p, float* ax, float* ay) {
    const float w = p[3];
    *ax = 1.f + p[0] / w;
    *ay = 1.f - p[1] / w;
}

void or_mark_edges(int H, int W, int B, int V, const float* pos, const int32_t* tri, int E,
                   const int32_t* edges, const int32_t* edge2tri, int32_t* prim_ids,
                   float* normals) {
    const float hh = (float)H * 0.5f, hw = (float)W * 0.5f;
#pragma omp parallel for schedule(static)
    for (int64_t idx = 0; idx < (int64_t)B * E; ++idx) {
        const int64_t b = idx / E, e = idx % E;
        const float* pb = pos + b * V * 4;
        const int v0 = edges[2 * e], v1 = edges[2 * e + 1];
        float ax0, ay0, ax1, ay1;
        proj_a(pb + (int64_t)v0 * 4, &ax0, &ay0);
        proj_a(pb + (int64_t)v1 * 4, &ax1, &ay1);
        const float x0 = hw * ax0, y0 = hh * ay0;
        const float dx = fmaf(hw, ax1, -x0), dy = fmaf(hh, ay1, -y0);
        const float len = sqrtf(fmaf(dx, dx, dy * dy));
        if (len == 0.f) continue;
        const float nx = -dy / len, ny = dx / len;
        float d0 = 0.f, d1 = 0.f;
        const int t0 = edge2tri[2 * e], t1 = edge2tri[2 * e + 1];
        if (t0 >= 0) {
            float ax2, ay2;
            proj_a(pb + (int64_t)third_vertex(tri, t0, v0, v1) * 4, &ax2, &ay2);
            d0 = dot2(nx, fmaf(hw, ax2, -x0), ny, fmaf(hh, ay2, -y0));
        }
        if (t1 >= 0) {
            float ax2, ay2;
            proj_a(pb + (int64_t)third_vertex(tri, t1, v0, v1) * 4, &ax2, &ay2);
            d1 = dot2(nx, fmaf(hw, ax2, -x0), ny, fmaf(hh, ay2, -y0));
        }
        if (d0 * d1 >= 0.f) prim_ids[idx] = (int32_t)idx;
        const float sign = 2.f * (.5f - (float)(d0 > 0.f || d1 > 0.f));
        normals[2 * idx] = sign * nx;
        normals[2 * idx + 1] = sign * ny;
    }
}

int64_t or_compact_ints(int64_t N, const int32_t* in, int32_t* out) {
    int64_t n = 0;
    for (int64_t i = 0; i < N; ++i)
        if (in[i] >= 0) out[n++] = in[i];
    return n;
}

static inline int bit_at(const int32_t* bits, int b, int w, int h, int c, int H, int W, int S) {
    const int64_t pix = (int64_t)H * W * b + w + (int64_t)h * W;
    return (bits[pix * S + c / 32] >> (c % 32)) & 1;
}

/* antialias.cu:121-176: FP32-mirrored window and disk decisions, FP64 weights */
static double adjoint_sum(int b, float x, float y, int c, int H, int W, int S,
                          const int32_t* bits, const int32_t* tgt, float kr, float rho) {
    const int R = f2i(floorf(kr));
    const int cw = f2i(floorf(x)), ch = f2i(floorf(y));
    const int h0 = imax(ch - R, 0), h1 = imin(ch + R, H - 1) + 1;
    const int w0 = imax(cw - R, 0), w1 = imin(cw + R, W - 1) + 1;
    const double sigma = (double)kr / 4.0;
    const double cc = 1.0 / (sigma * sigma * 2.0 * 3.14159265358979323846);
    const double alpha = 0.5 / (sigma * sigma);
    double dc = 0.0;
    for (int h = h0; h < h1; ++h)
        for (int w = w0; w < w1; ++w) {
            const int c0 = bit_at(bits, b, w, h, c, H, W, S);
            const int c1 = bit_at(tgt, b, w, h, c, H, W, S);
            if (c0 == c1) continue;
            const float dx = (float)w + 0.5f - x, dy = (float)h + 0.5f - y;
            const float n2 = dot2(dx, dx, dy, dy);
            if (!(n2 < kr * kr)) continue;
            const double n2d = (double)dx * dx + (double)dy * dy;
            dc += cc * exp(-alpha * n2d) * (double)(c0 - c1) * (c1 == 0 ? (double)rho : 1.0);
        }
    return dc;
}

/* antialias.cu:179-279 */
void or_aa_backward(int64_t F, const int32_t* frag_pix, const float* frag_attrs, int H, int W,
                    int S, const int32_t* bitset, const int32_t* target, int V,
                    const float* pos, int E, const int32_t* edges, const float* normals,
                    const int32_t* edge2cluster, double* d_pos, float kernel_radius, float rho,
                    double* frag_dc) {
    const float fH = (float)H, fW = (float)W;
    for (int64_t i = 0; i < F; ++i) {
        if (frag_dc) frag_dc[i] = 0.0;
        const int b = frag_pix[3 * i], h = frag_pix[3 * i + 1], w = frag_pix[3 * i + 2];
        const float axis = frag_attrs[4 * i], t1 = frag_attrs[4 * i + 1], t0 = 1.f - t1;
        const int e = f2i(frag_attrs[4 * i + 3]) - 1;
        if (e < 0) continue;
        const float* pb = pos + (int64_t)b * V * 4;
        const int v0 = edges[2 * e], v1 = edges[2 * e + 1];
        const float p0x = pb[v0 * 4], p0y = pb[v0 * 4 + 1], p0w = pb[v0 * 4 + 3];
        const float p1x = pb[v1 * 4], p1y = pb[v1 * 4 + 1], p1w = pb[v1 * 4 + 3];
        const float px = dot2(t0, p0x, t1, p1x);
        const float py = dot2(t0, p0y, t1, p1y);
        const float pw = dot2(t0, p0w, t1, p1w);
        const float fx = 0.5f * (1.f + px / pw) * fW;
        const float fy = 0.5f * (1.f - py / pw) * fH;
        const float nx = normals[(int64_t)b * E * 2 + 2 * e], ny = normals[(int64_t)b * E * 2 + 2 * e + 1];
        int nh = h, nw = w;
        const float rx = fx - floorf(fx), ry = fy - floorf(fy);
        const float eps = 1e-4f;
        float dot = 0.f;
        if (axis == 0.f) {
            if (!isfinite(rx) || fabsf(rx - 0.5f) >= eps) continue;
            const int d = 2 * (int)(ry > 0.5f) - 1;
            nh += d;
            dot += (float)d * ny;
        } else {
            if (!isfinite(ry) || fabsf(ry - 0.5f) >= eps) continue;
            const int d = 2 * (int)(rx > 0.5f) - 1;
            nw += d;
            dot += (float)d * nx;
        }
        if (nw < 0 || nw >= W || nh < 0 || nh >= H || dot == 0.f) continue;
        const int c = edge2cluster[e];
        const double c01 = dot > 0.f ? 1.0 - bit_at(bitset, b, nw, nh, c, H, W, S)
                                     : 1.0 - bit_at(bitset, b, w, h, c, H, W, S);
        if (c01 == 0.0) continue;
        const double dc = c01 * adjoint_sum(b, fx, fy, c, H, W, S, bitset, target, kernel_radius, rho);
        if (dc == 0.0) continue;
        if (frag_dc) frag_dc[i] = dc;
        const double dx = dc * 0.5 * fW * nx;
        const double dy = dc * -0.5 * fH * ny;
        const double dpx = dx / pw, dpy = dy / pw;
        const double dpw = (dx * px + dy * py) / ((double)pw * pw);
        if (!isfinite(dpx) || !isfinite(dpy) || !isfinite(dpw)) continue;
        double* g0 = d_pos + ((int64_t)b * V + v0) * 4;
        double* g1 = d_pos + ((int64_t)b * V + v1) * 4;
        g0[0] += dpx * t0; g0[1] += dpy * t0; g0[3] += dpw * t0;
        g1[0] += dpx * t1; g1[1] += dpy * t1; g1[3] += dpw * t1;
    }
}

/* ================================================================================== */
/* bitset utils (bitset_utils.cu)                                                      */
/* ================================================================================== */

void or_popcount(int64_t npix, int S, const int32_t* bitset, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        int n = 0;
        for (int s = 0; s < S; ++s) n += __builtin_popcount((uint32_t)bitset[p * S + s]);
        out[p] = (float)n;
    }
}

/* bitset_utils.cu:6-35: same summation order, so FP32 results are bit-identical */
void or_accumulate_rgb(int64_t npix, int S, const int32_t* bitset, const float* rgb, float* out) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        float r = 0.f, g = 0.f, bb = 0.f;
        for (int s = 0; s < S; ++s) {
            const uint32_t m = (uint32_t)bitset[p * S + s];
            if (!m) continue;
            for (int j = 0; j < 32; ++j)
                if (m & (1u << j)) {
                    const int c = s * 32 + j;
                    r += rgb[c * 3]; g += rgb[c * 3 + 1]; bb += rgb[c * 3 + 2];
                }
        }
        out[3 * p] = r; out[3 * p + 1] = g; out[3 * p + 2] = bb;
    }
}

/* ================================================================================== */
/* curves (curve_utils.cu), FP64 with the FP32 cutoff decision                          */
/* ================================================================================== */

void or_smooth_strands(int N, int V, const float* strands, const float* arclength,
                       double* out, float beta) {
    const float cutoff = 3.0f * beta;
    const double ib2 = 1.0 / ((double)beta * beta);
#pragma omp parallel for schedule(static)
    for (int s = 0; s < N; ++s) {
        const float* arc = arclength + (int64_t)s * V;
        const float* x = strands + (int64_t)s * V * 3;
        for (int i = 0; i < V; ++i) {
            double acc[3] = {0, 0, 0}, sw = 0.0;
            for (int j = 0; j < V; ++j) {
                const float dist = fabsf(arc[i] - arc[j]);
                if (dist > cutoff) continue;
                const double w = exp(-(double)dist * dist * ib2);
                acc[0] += w * x[3 * j]; acc[1] += w * x[3 * j + 1]; acc[2] += w * x[3 * j + 2];
                sw += w;
            }
            double* o = out + ((int64_t)s * V + i) * 3;
            if (sw > 1e-6) { o[0] = acc[0] / sw; o[1] = acc[1] / sw; o[2] = acc[2] / sw; }
            else { o[0] = o[1] = o[2] = 0.0; }
        }
    }
}

void or_skinning(int N, int V, const float* strands, const float* arclength,
                 const float* handles, const float* canonical, const float* R,
                 double* out, float beta) {
    const float cutoff = 3.0f * beta;
    const double ib2 = 1.0 / ((double)beta * beta);
#pragma omp parallel for schedule(static)
    for (int s = 0; s < N; ++s) {
        const int64_t o3 = (int64_t)s * V * 3;
        const float* arc = arclength + (int64_t)s * V;
        for (int i = 0; i < V; ++i) {
            double acc[3] = {0, 0, 0}, sw = 0.0;
            for (int j = 0; j < V; ++j) {
                const float dist = fabsf(arc[i] - arc[j]);
                if (dist > cutoff) continue;
                const double w = exp(-(double)dist * dist * ib2);
                double l[3];
                for (int k = 0; k < 3; ++k) l[k] = (double)strands[o3 + 3 * i + k] - handles[o3 + 3 * j + k];
                const float* Rj = R + ((int64_t)s * V + j) * 9;
                for (int r = 0; r < 3; ++r)
                    acc[r] += w * (Rj[3 * r] * l[0] + Rj[3 * r + 1] * l[1] + Rj[3 * r + 2] * l[2] +
                                   canonical[o3 + 3 * j + r]);
                sw += w;
            }
            double* o = out + o3 + 3 * i;
            if (sw > 1e-8) { o[0] = acc[0] / sw; o[1] = acc[1] / sw; o[2] = acc[2] / sw; }
            else { o[0] = strands[o3 + 3 * i]; o[1] = strands[o3 + 3 * i + 1]; o[2] = strands[o3 + 3 * i + 2]; }
        }
    }
}

/* 4 nearest guides of each vertex by brute force, for the GPU binding of linear blend
 * skinning: d^2 = (dx*dx + dy*dy) + dz*dz in FP32 (no contraction), ties to the lower
 * guide index, non-finite distances never selected; idx = -1 / d2 = +inf where fewer
 * than 4 guides qualify. */
void or_knn4(int64_t Nv, const float* x, int G, const float* g, int32_t* idx, float* d2) {
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < Nv; ++v) {
        float bd[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
        int bi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
        const float qx = x[3 * v], qy = x[3 * v + 1], qz = x[3 * v + 2];
        for (int i = 0; i < G; ++i) {
            const float dx = qx - g[3 * i], dy = qy - g[3 * i + 1], dz = qz - g[3 * i + 2];
            const float sx = dx * dx, sy = dy * dy, sz = dz * dz;
            const float s = (sx + sy) + sz;
            if (!(s < bd[3] || (s == bd[3] && i < bi[3]))) continue;
            int k = 3;
            while (k > 0 && (s < bd[k - 1] || (s == bd[k - 1] && i < bi[k - 1]))) {
                bd[k] = bd[k - 1];
                bi[k] = bi[k - 1];
                --k;
            }
            bd[k] = s;
            bi[k] = i;
        }
        for (int k = 0; k < 4; ++k) {
            const int ok = bi[k] != 0x7fffffff && isfinite(bd[k]);
            idx[4 * v + k] = ok ? bi[k] : -1;
            d2[4 * v + k] = ok ? bd[k] : INFINITY;
        }
    }
}
