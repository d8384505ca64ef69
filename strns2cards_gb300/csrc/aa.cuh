// Antialias helpers shared by the antialias kernels and the batched fit kernel: the
// silhouette test with its oriented normal (antialias.cu:38-94), the Gaussian window
// constants (antialias.cu:121-131), the chain rule (antialias.cu:281-316) and compensated
// FP32 sums.  Vertex positions come through an accessor, so the same arithmetic runs on
// global or shared-memory copies.
#pragma once
#include "common.cuh"

namespace s2c {

__device__ __forceinline__ int third_vertex(const int* __restrict__ tri, int t, int v0, int v1) {
    const int i0 = __ldg(tri + 3 * t), i1 = __ldg(tri + 3 * t + 1), i2 = __ldg(tri + 3 * t + 2);
    return (i0 != v0 && i0 != v1) ? i0 : (i1 != v0 && i1 != v1) ? i1 : (i2 != v0 && i2 != v1) ? i2 : -1;
}

// antialias.cu:29-35 without the final multiply: (1 + x/w, 1 - y/w)
__device__ __forceinline__ float2 ndc_a(float4 p) {
    return make_float2(__fadd_rn(1.f, __fdiv_rn(p.x, p.w)), __fsub_rn(1.f, __fdiv_rn(p.y, p.w)));
}

// antialias.cu:38-94 for edge ev with adjacent triangles tt (-1 = none); pos(v) gives vertex
// v of the view: 0 = zero-length edge (no normal), 1 = normal only, 2 = silhouette or
// boundary edge (marked) with its oriented normal
template <class PosF>
__device__ __forceinline__ int mark_edge_t(int H, int W, int2 ev, int2 tt, const int* __restrict__ tri, int T, int V,
                                           PosF pos, float2& nrm) {
    if ((unsigned)ev.x >= (unsigned)V || (unsigned)ev.y >= (unsigned)V) return 0;
    const float hh = __fmul_rn((float)H, 0.5f), hw = __fmul_rn((float)W, 0.5f);
    const float2 a0 = ndc_a(pos(ev.x)), a1 = ndc_a(pos(ev.y));
    const float x0 = __fmul_rn(hw, a0.x), y0 = __fmul_rn(hh, a0.y);
    const float dx = __fmaf_rn(hw, a1.x, -x0), dy = __fmaf_rn(hh, a1.y, -y0);
    const float len = __fsqrt_rn(__fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
    if (len == 0.f) return 0;
    const float nx = __fdiv_rn(-dy, len), ny = __fdiv_rn(dx, len);
    float d[2] = {0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int t = i ? tt.y : tt.x;
        if (t < 0 || t >= T) continue;
        const int v2 = third_vertex(tri, t, ev.x, ev.y);
        if ((unsigned)v2 >= (unsigned)V) continue;  // degenerate triangle (the reference reads out of bounds)
        const float2 a2 = ndc_a(pos(v2));
        d[i] = __fmaf_rn(nx, __fmaf_rn(hw, a2.x, -x0), __fmul_rn(ny, __fmaf_rn(hh, a2.y, -y0)));
    }
    const float sign = __fmul_rn(2.f, __fsub_rn(0.5f, (float)(d[0] > 0.f || d[1] > 0.f)));
    nrm = make_float2(__fmul_rn(sign, nx), __fmul_rn(sign, ny));
    return __fmul_rn(d[0], d[1]) >= 0.f ? 2 : 1;
}

// Compensated FP32 sums (no FP64 arithmetic on the SMs: GB300's FP64 rate is a small
// fraction of its FP32 rate).  kahan_add: running (sum, comp); two_sum_merge: error-free
// merge of two compensated sums (Knuth's 2Sum on the leading parts).
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
    const float y = __fsub_rn(v, comp);
    const float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

__device__ __forceinline__ void two_sum_merge(float& hi, float& lo, float ohi, float olo) {
    const float s = __fadd_rn(hi, ohi);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(ohi, bb));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, olo), err);
}

// warp-wide compensated sum of the lanes' (sum, -comp) pairs, rounded to float
__device__ __forceinline__ float warp_sum_comp(float sum, float comp) {
    float hi = sum, lo = -comp;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        const float ohi = __shfl_xor_sync(0xffffffffu, hi, off), olo = __shfl_xor_sync(0xffffffffu, lo, off);
        two_sum_merge(hi, lo, ohi, olo);
    }
    return __fadd_rn(hi, lo);
}

// Border rows / columns of a window whose offset alone reaches the disk's edge hold no
// pixel with n2 = fma(dx, dx, dy * dy) < kr^2 (n2 >= fl(dy * dy) and n2 >= fl(dx * dx), with
// d = (t + 0.5) - f as the window sums compute it): dropping them changes no sum.  With the
// half-pixel test, one axis's offsets are whole numbers and its two border lines sit exactly
// on the edge.
__device__ __forceinline__ float aa_off2(int t, float f) {
    const float d = __fsub_rn(__fadd_rn((float)t, 0.5f), f);
    return __fmul_rn(d, d);
}

__device__ __forceinline__ void aa_trim_window(float kr, float fx, float fy, int& h0, int& h1, int& w0, int& w1) {
    const float kr2 = __fmul_rn(kr, kr);
    while (h0 < h1 && !(aa_off2(h0, fy) < kr2)) ++h0;
    while (h1 > h0 && !(aa_off2(h1 - 1, fy) < kr2)) --h1;
    while (w0 < w1 && !(aa_off2(w0, fx) < kr2)) ++w0;
    while (w1 > w0 && !(aa_off2(w1 - 1, fx) < kr2)) --w1;
}

// Gaussian window constants of antialias.cu:121-131
struct AAWin {
    float cc, alpha, kr2;
};

__device__ __forceinline__ AAWin aa_win(float kr) {
    AAWin q;
    const float sigma = __fdiv_rn(kr, 4.f);
    q.cc = __fdiv_rn(1.f, __fmul_rn(__fmul_rn(__fmul_rn(sigma, sigma), 2.f), 3.14159265358979323846f));
    q.alpha = __fdiv_rn(0.5f, __fmul_rn(sigma, sigma));
    q.kr2 = __fmul_rn(kr, kr);
    return q;
}

// Chain rule of one fragment in FP32 (antialias.cu:281-316): (d/dx, d/dy, d/dw) of the edge
// point (px, py, pw) from the window sum dc and the edge normal; false if not finite
__device__ __forceinline__ bool aa_chain_rule(int H, int W, float dc, float2 nrm, float px, float py, float pw,
                                              float& dpx, float& dpy, float& dpw) {
    const float dx = __fmul_rn(__fmul_rn(__fmul_rn(dc, 0.5f), (float)W), nrm.x);
    const float dy = __fmul_rn(__fmul_rn(__fmul_rn(dc, -0.5f), (float)H), nrm.y);
    dpx = __fdiv_rn(dx, pw);
    dpy = __fdiv_rn(dy, pw);
    dpw = __fdiv_rn(__fmaf_rn(dx, px, __fmul_rn(dy, py)), __fmul_rn(pw, pw));
    return isfinite(dpx) && isfinite(dpy) && isfinite(dpw);
}

}  // namespace s2c
