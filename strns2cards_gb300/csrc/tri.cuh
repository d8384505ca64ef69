// Triangle coverage arithmetic shared by the raster kernels and the batched fit kernel:
// the reference's FP32 formulas (rasterize.cu:9-172) with its fusion shapes, so coverage,
// barycentrics and depth are bit-identical to it.  Positions come in as loaded values, so
// the same code serves global and shared-memory copies of the corners.
#pragma once
#include "common.cuh"

namespace s2c {

// rasterize.cu:9-59: screen rectangle (h0, h_len, w0, w_len) of a triangle from its three
// clip-space corners; ok[i] = false marks a corner whose vertex index was out of range (the
// reference would read out of bounds): the rectangle is then empty
__device__ __forceinline__ int4 tri_rect_of(int H, int W, const float4 (&P)[3], const bool (&ok)[3]) {
    const float fH = (float)H, fW = (float)W;
    float x0 = fW, y0 = fH, x1 = 0.f, y1 = 0.f;
    bool bad = false;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (!ok[i]) { bad = true; continue; }
        const float4 p = P[i];
        const float inv_w = __fdiv_rn(1.f, p.w);
        const float x = __fmul_rn(__fmul_rn(0.5f, __fmaf_rn(p.x, inv_w, 1.f)), fW);
        const float y = __fmul_rn(__fmul_rn(0.5f, __fmaf_rn(-p.y, inv_w, 1.f)), fH);
        x0 = isnan(x) ? x0 : fminf(x, x0);
        x1 = isnan(x) ? x1 : fmaxf(x, x1);
        y0 = isnan(y) ? y0 : fminf(y, y0);
        y1 = isnan(y) ? y1 : fmaxf(y, y1);
    }
    const int h0 = max(f2i(floorf(y0)), 0);
    const int h1 = min(f2i(floorf(y1)), H - 1) + 1;
    const int w0 = max(f2i(floorf(x0)), 0);
    const int w1 = min(f2i(floorf(x1)), W - 1) + 1;
    int hl = (int)((unsigned)h1 - (unsigned)h0), wl = (int)((unsigned)w1 - (unsigned)w0);
    hl = hl > 0 ? hl : 0;
    wl = wl > 0 ? wl : 0;
    if (bad) hl = wl = 0;
    return make_int4(h0, hl, w0, wl);
}

// Pixel centre in NDC (rasterize.cu:132-133)
__device__ __forceinline__ float ndc_of(int i, float n) {
    return __fadd_rn(-1.f, __fdiv_rn(__fmul_rn(2.f, __fadd_rn((float)i, 0.5f)), n));
}

// Clip-space edge functions of a pixel centre (rasterize.cu:140-150)
struct TriEdges {
    float A0, A1, A2, A;
};

__device__ __forceinline__ TriEdges tri_edges(float4 P0, float4 P1, float4 P2, float px, float py) {
    const float q0x = __fmaf_rn(-px, P0.w, P0.x), q0y = __fmaf_rn(-py, P0.w, -P0.y);
    const float q1x = __fmaf_rn(-px, P1.w, P1.x), q1y = __fmaf_rn(-py, P1.w, -P1.y);
    const float q2x = __fmaf_rn(-px, P2.w, P2.x), q2y = __fmaf_rn(-py, P2.w, -P2.y);
    TriEdges e;
    // a*b - c*d is fused on its first product
    e.A0 = __fmaf_rn(q1x, q2y, -__fmul_rn(q1y, q2x));
    e.A1 = __fmaf_rn(q2x, q0y, -__fmul_rn(q2y, q0x));
    e.A2 = __fmaf_rn(q0x, q1y, -__fmul_rn(q0y, q1x));
    e.A = __fadd_rn(__fadd_rn(e.A0, e.A1), e.A2);
    return e;
}

// rasterize.cu:151-163: barycentrics, depth and the acceptance test
__device__ __forceinline__ bool tri_finish(const TriEdges& e, float4 P0, float4 P1, float4 P2, float& b0, float& b1,
                                           float& z) {
    if (e.A == 0.f) return false;
    const float invA = __fdiv_rn(1.f, e.A);
    b0 = __fmul_rn(e.A0, invA);
    b1 = __fmul_rn(e.A1, invA);
    // the barycentric half of the acceptance test first: the depth division only for
    // pixels that pass it (the conjunction, and so the result, is the same)
    if (!isfinite(b0) || !isfinite(b1) || b0 < 0.f || b1 < 0.f || __fadd_rn(b0, b1) > 1.f) return false;
    // (A0 z0 + A1 z1) + A2 z2 and the same for w, with the reference build's fusion shapes
    const float zc = __fmaf_rn(e.A2, P2.z, __fmaf_rn(e.A1, P1.z, __fmul_rn(e.A0, P0.z)));
    const float wc = __fmaf_rn(e.A2, P2.w, __fmaf_rn(e.A0, P0.w, __fmul_rn(e.A1, P1.w)));
    z = __fdiv_rn(zc, wc);
    if (!isfinite(z) || z < -1.f || z > 1.f) return false;
    return true;
}

// Coverage of pixel (x, y) by a triangle with clip-space corners P0..P2
// (rasterize.cu:132-163).  Returns true and (b0, b1, z) when covered.
__device__ __forceinline__ bool tri_cover(int H, int W, float4 P0, float4 P1, float4 P2, int x, int y, float& b0,
                                          float& b1, float& z) {
    const TriEdges e = tri_edges(P0, P1, P2, ndc_of(x, (float)W), ndc_of(y, (float)H));
    return tri_finish(e, P0, P1, P2, b0, b1, z);
}

// Exact early rejection: with A and A_i finite, opposite signs and |A_i| > 1e-30 |A|, the
// product A_i * fl(1 / A) is a nonzero number of A_i's sign * sign(A) (no underflow), so
// b_i < 0 and tri_finish rejects the pixel.
__device__ __forceinline__ bool tri_surely_outside(const TriEdges& e) {
    if (!isfinite(e.A) || e.A == 0.f) return e.A == 0.f;
    const float lim = __fmul_rn(fabsf(e.A), 1e-30f);
    const bool out0 = isfinite(e.A0) && e.A0 != 0.f && ((e.A0 < 0.f) != (e.A < 0.f)) && fabsf(e.A0) > lim;
    const bool out1 = isfinite(e.A1) && e.A1 != 0.f && ((e.A1 < 0.f) != (e.A < 0.f)) && fabsf(e.A1) > lim;
    return out0 || out1;
}

}  // namespace s2c
