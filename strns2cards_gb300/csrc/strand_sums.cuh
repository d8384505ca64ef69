// Per-strand pieces shared by the curve kernels (curves.cu) and the fused wisp alignment
// (frames.cu), so that both give the same bits: the in-kernel arclength (a warp scan) and
// the Gaussian-in-arclength sums of smoothing and skinning for one point (the reference's
// curve_utils.cu:24-68 and :70-131 loop bodies).
#pragma once

#include <cuda_runtime.h>

namespace s2c {

// arclength of one strand (points x[0..V), xyz interleaved) into arc[0..V), by one warp:
// segment lengths, then an inclusive warp scan per 32-point chunk carried across chunks.
// The scan's sums take different rounding paths per lane; a running maximum (exact, and a
// NaN stays NaN) keeps the result non-decreasing, which strand_pair_window relies on.
__device__ __forceinline__ void warp_arclength(const float* x, int V, float* arc, int lane) {
    float carry = 0.f;
    for (int base = 0; base < V; base += 32) {
        const int i = base + lane;
        float d = 0.f;
        if (i > 0 && i < V) {
            const float dx = __fsub_rn(x[3 * i], x[3 * i - 3]);
            const float dy = __fsub_rn(x[3 * i + 1], x[3 * i - 2]);
            const float dz = __fsub_rn(x[3 * i + 2], x[3 * i - 1]);
            d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_up_sync(0xffffffffu, d, o);
            if (lane >= o) d = __fadd_rn(d, t);
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_up_sync(0xffffffffu, d, o);
            if (lane >= o && t > d) d = t;
        }
        if (i < V) arc[i] = __fadd_rn(carry, d);
        carry = __fadd_rn(carry, __shfl_sync(0xffffffffu, d, 31));
    }
}

// The j range of the pair sums of point i.  With a non-decreasing arclength (the one
// warp_arclength computes) the points within the cutoff form one run around i: walk out to
// its ends.  Otherwise (a caller's arclength, or a non-finite one) all of 0..V-1.  Every j
// in the range is still tested against the cutoff, so the sums have the same terms in the
// same order as the full loop.
__device__ __forceinline__ void strand_pair_window(const float* arc, int V, int i, float cutoff, bool monotone,
                                                   int& jlo, int& jhi) {
    jlo = 0;
    jhi = V - 1;
    const float si = arc[i];
    if (monotone && isfinite(si) && isfinite(arc[V - 1])) {
        jlo = i;
        while (jlo > 0 && !(fabsf(__fsub_rn(si, arc[jlo - 1])) > cutoff)) --jlo;
        jhi = i;
        while (jhi < V - 1 && !(fabsf(__fsub_rn(si, arc[jhi + 1])) > cutoff)) ++jhi;
    }
}

// smooth_strands for point i: sum_j w_ij x_j / sum_j w_ij, w = exp(-d^2 / beta^2) over
// |a_i - a_j| <= cutoff; 0 where the weight sum is <= 1e-6
__device__ __forceinline__ void smooth_point(const float* X, const float* arc, int V, int i, float cutoff,
                                             float inv_beta2, bool monotone, float out[3]) {
    int jlo, jhi;
    strand_pair_window(arc, V, i, cutoff, monotone, jlo, jhi);
    const float si = arc[i];
    float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, sw = 0.f;
    for (int j = jlo; j <= jhi; ++j) {
        const float dist = fabsf(__fsub_rn(si, arc[j]));
        if (dist > cutoff) continue;
        const float w = expf(__fmul_rn(-__fmul_rn(dist, dist), inv_beta2));
        acc0 = __fmaf_rn(w, X[3 * j], acc0);
        acc1 = __fmaf_rn(w, X[3 * j + 1], acc1);
        acc2 = __fmaf_rn(w, X[3 * j + 2], acc2);
        sw = __fadd_rn(sw, w);
    }
    const bool ok = sw > 1e-6f;
    out[0] = ok ? __fdiv_rn(acc0, sw) : 0.f;
    out[1] = ok ? __fdiv_rn(acc1, sw) : 0.f;
    out[2] = ok ? __fdiv_rn(acc2, sw) : 0.f;
}

// skinning for point i: sum_j w_ij (R_j (x_i - h_j) + c_j) / sum_j w_ij; x_i where the
// weight sum is <= 1e-8.  R row-major 3x3 per point.
__device__ __forceinline__ void skin_point(const float* X, const float* arc, const float* Hh, const float* Cc,
                                           const float* RR, int V, int i, float cutoff, float inv_beta2,
                                           bool monotone, float out[3]) {
    int jlo, jhi;
    strand_pair_window(arc, V, i, cutoff, monotone, jlo, jhi);
    const float si = arc[i];
    const float xi0 = X[3 * i], xi1 = X[3 * i + 1], xi2 = X[3 * i + 2];
    float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, sw = 0.f;
    for (int j = jlo; j <= jhi; ++j) {
        const float dist = fabsf(__fsub_rn(si, arc[j]));
        if (dist > cutoff) continue;
        const float w = expf(__fmul_rn(-__fmul_rn(dist, dist), inv_beta2));
        const float l0 = __fsub_rn(xi0, Hh[3 * j]);
        const float l1 = __fsub_rn(xi1, Hh[3 * j + 1]);
        const float l2 = __fsub_rn(xi2, Hh[3 * j + 2]);
        const float* r = RR + 9 * j;
        const float r0 = __fmaf_rn(r[2], l2, __fmaf_rn(r[1], l1, __fmul_rn(r[0], l0)));
        const float r1 = __fmaf_rn(r[5], l2, __fmaf_rn(r[4], l1, __fmul_rn(r[3], l0)));
        const float r2 = __fmaf_rn(r[8], l2, __fmaf_rn(r[7], l1, __fmul_rn(r[6], l0)));
        acc0 = __fmaf_rn(w, __fadd_rn(r0, Cc[3 * j]), acc0);
        acc1 = __fmaf_rn(w, __fadd_rn(r1, Cc[3 * j + 1]), acc1);
        acc2 = __fmaf_rn(w, __fadd_rn(r2, Cc[3 * j + 2]), acc2);
        sw = __fadd_rn(sw, w);
    }
    const bool ok = sw > 1e-8f;
    out[0] = ok ? __fdiv_rn(acc0, sw) : xi0;
    out[1] = ok ? __fdiv_rn(acc1, sw) : xi1;
    out[2] = ok ? __fdiv_rn(acc2, sw) : xi2;
}

}  // namespace s2c
