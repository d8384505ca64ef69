// Strand frames and wisp alignment (the reference's curve_utils.py:9-165 and 243-308:
// minimal_rotation, tangent_frame, compute_bishop_frame, compute_aligned_strands,
// compute_alignment_rotation; and align_wisps, :481-607).
//
// The reference runs the Bishop (rotation-minimising) frame recurrence as a Python loop
// over the points of all strands and the wisp frames as a Python loop over wisps with a
// host SVD each.  Here:
//   strand_frames_kernel  one warp per strand, one lane per point: the recurrence as a warp
//                         scan of 3x3 maps (frame_chunk), frames, alignment rotations and
//                         canonical handles in one pass;
//   wisp_frames_kernel    one CTA per wisp: root centre, longest strand, FP32 second moment
//                         of the centred roots and a cyclic Jacobi eigen-solve in place of
//                         the SVD (the least-variance axis is the singular vector the frame
//                         uses), the wisp's rotation;
//   wisp_rotate_kernel    the strands and handles turned into their wisp's frame;
//   align_strands_kernel  smoothing, rotation, frames and skinning of each strand fused
//                         (one warp per strand staged in shared memory), with the same
//                         device code as the separate steps.
// FP32 throughout, with the reference's formulas.
#include <algorithm>

#include "common.cuh"
#include "strand_sums.cuh"

namespace s2c {
namespace {

struct V3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm(V3 a) { return sqrtf(dot(a, a)); }
// v / max(|v|, 1e-8)
__device__ __forceinline__ V3 unit(V3 a) { return mul(a, 1.f / fmaxf(norm(a), 1e-8f)); }
__device__ __forceinline__ V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float* p, V3 a) {
    p[0] = a.x;
    p[1] = a.y;
    p[2] = a.z;
}

// tangent_frame (curve_utils.py:76-102): branch-free orthonormal basis around t
__device__ __forceinline__ void tangent_frame(V3 t, V3& n, V3& b) {
    t = unit(t);
    const float sign = t.z > 0.f ? 1.f : (t.z < 0.f ? -1.f : 1.f);
    const float a = -1.f / (sign + t.z);
    const float bb = t.x * t.y * a;
    n = v3(1.f + sign * t.x * t.x * a, sign * bb, -sign * t.x);
    b = v3(bb, sign + t.y * t.y * a, -t.y);
}

// minimal_rotation (curve_utils.py:9-74): the rotation taking src to dst (Rodrigues), row-major
__device__ __forceinline__ void minimal_rotation(V3 s, V3 d, float R[9]) {
    s = unit(s);
    d = unit(d);
    V3 ax = cross(s, d);
    const float sin_t = norm(ax);
    const float cos_t = fminf(fmaxf(dot(s, d), -1.f), 1.f);
    ax = mul(ax, 1.f / fmaxf(sin_t, 1e-8f));
    for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? 1.f : 0.f;
    if (cos_t > 1.f - 1e-6f) return;
    if (cos_t < -1.f + 1e-6f) {
        R[0] = -1.f;
        R[4] = -1.f;
        R[8] = 1.f;
        return;
    }
    const float K[9] = {0.f, -ax.z, ax.y, ax.z, 0.f, -ax.x, -ax.y, ax.x, 0.f};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            float kk = 0.f;
            for (int k = 0; k < 3; ++k) kk += K[3 * r + k] * K[3 * k + c];
            R[3 * r + c] += sin_t * K[3 * r + c] + (1.f - cos_t) * kk;
        }
}

__device__ __forceinline__ V3 matvec(const float R[9], V3 v) {
    return v3(R[0] * v.x + R[1] * v.y + R[2] * v.z, R[3] * v.x + R[4] * v.y + R[5] * v.z,
              R[6] * v.x + R[7] * v.y + R[8] * v.z);
}

// tangent of point i: (p[i+1] - p[i]) + (p[i] - p[i-1]), one-sided at the ends, normalised
__device__ __forceinline__ V3 tangent_at(const float* p, int i, int V) {
    V3 t = v3(0.f, 0.f, 0.f);
    if (i + 1 < V) t = add(t, sub(ld3(p + 3 * (i + 1)), ld3(p + 3 * i)));
    if (i > 0) t = add(t, sub(ld3(p + 3 * i), ld3(p + 3 * (i - 1))));
    return unit(t);
}


// 3x3 row-major helpers for the frame scan
struct M3 {
    float m[9];
};
__device__ __forceinline__ M3 m3_identity() {
    M3 r;
#pragma unroll
    for (int k = 0; k < 9; ++k) r.m[k] = (k % 4 == 0) ? 1.f : 0.f;
    return r;
}
// The scan's own arithmetic (not an operation order of the reference's) uses fused
// multiply-adds: a third of the instructions of separate products and sums.
__device__ __forceinline__ M3 m3_mul(const M3& A, const M3& B) {
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] =
                __fmaf_rn(A.m[3 * i + 2], B.m[6 + j], __fmaf_rn(A.m[3 * i + 1], B.m[3 + j], A.m[3 * i] * B.m[j]));
    return r;
}
__device__ __forceinline__ V3 m3_vec(const M3& A, V3 v) {
    return v3(__fmaf_rn(A.m[2], v.z, __fmaf_rn(A.m[1], v.y, A.m[0] * v.x)),
              __fmaf_rn(A.m[5], v.z, __fmaf_rn(A.m[4], v.y, A.m[3] * v.x)),
              __fmaf_rn(A.m[8], v.z, __fmaf_rn(A.m[7], v.y, A.m[6] * v.x)));
}
// I - k v v^T
__device__ __forceinline__ M3 householder(V3 v, float k) {
    M3 r;
    const float c[3] = {v.x, v.y, v.z};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float kc = -k * c[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = __fmaf_rn(kc, c[j], i == j ? 1.f : 0.f);
    }
    return r;
}
__device__ __forceinline__ V3 shfl_up3(V3 v, int d) {
    return v3(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
              __shfl_up_sync(0xffffffffu, v.z, d));
}
__device__ __forceinline__ V3 shfl3(V3 v, int src) {
    return v3(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
              __shfl_sync(0xffffffffu, v.z, src));
}

// `C` values per lane for 32 consecutive items -> dst[0 .. nitems*C), through buf (32*C floats),
// so that each store instruction of the warp writes a contiguous run
template <int C>
__device__ __forceinline__ void warp_store(float* buf, const float (&v)[C], float* __restrict__ dst, int nitems,
                                           int lane) {
#pragma unroll
    for (int c = 0; c < C; ++c) buf[lane * C + c] = v[c];
    __syncwarp();
    for (int f = lane; f < nitems * C; f += 32) dst[f] = buf[f];
    __syncwarp();
}

struct FrameArgs {
    int64_t N;
    int V;
    const float* strands;   // (N, V, 3)
    V3 tdst;
    float* T;               // (N, V, 3) nullable
    float* Nn;              // nullable
    float* Bn;              // nullable
    float* R;               // (N, V, 3, 3) nullable: compute_alignment_rotation
    const float* roots;     // nullable: compute_aligned_strands roots (else the strands' own first points)
    int64_t roots_stride;   // floats between consecutive roots
    float* canon;           // (N, V, 3) nullable: compute_aligned_strands
};

constexpr int kFrameThreads = 256;
constexpr int kFrameWarps = kFrameThreads / 32;

__device__ __forceinline__ V3 shfl_down3(V3 v, int d) {
    return v3(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
              __shfl_down_sync(0xffffffffu, v.z, d));
}
__device__ __forceinline__ float shfl_f(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// State a warp carries from one 32-point chunk of a strand to the next.
struct FrameCarry {
    V3 n0, b0;       // the root frame (tangent_frame of the root tangent)
    V3 nd, bd;       // the root frame turned onto t_dst (minimal rotation)
    V3 n_prev;       // the normal at the point before the chunk
    V3 p_last, t_last;
    float arc;       // arclength at the point before the chunk
};

struct FramePoint {
    V3 p, t, n, b;
    float arc;
};

__device__ __forceinline__ void frame_root(const float* p, int V, V3 td, bool want_dst, FrameCarry& cy) {
    const V3 t0 = tangent_at(p, 0, V);
    tangent_frame(t0, cy.n0, cy.b0);
    cy.nd = cy.n0;
    cy.bd = cy.b0;
    if (want_dst) {
        float Ra[9];
        minimal_rotation(t0, td, Ra);
        cy.nd = matvec(Ra, cy.n0);
        cy.bd = matvec(Ra, cy.b0);
    }
    cy.n_prev = cy.n0;
    cy.p_last = ld3(p);
    cy.t_last = t0;
    cy.arc = 0.f;
}

// One 32-point chunk (points c0 + lane) of the rotation-minimising frame of the strand p
// (curve_utils.py:104-165), for the whole warp.  The reference steps the normal point by
// point: n_i = normalize(H2_i H1_i n_{i-1}), H1_i = I - 2 v1 v1^T / c1 (v1 = x_i - x_{i-1}) and
// H2_i = I - 2 v2 v2^T / c2 (v2 = t_i - H1_i t_{i-1}), c clamped below at 1e-8.  Neither map
// depends on the normal and each normalisation only scales by a positive number, so
// n_i = normalize(M_i ... M_c0 n_{c0-1}) with M_i = H2_i H1_i: every lane builds its M_i and
// a warp scan forms the prefix products (later factors on the left).  Tangents as the
// reference's (x_{i+1} - x_i) + (x_i - x_{i-1}), one-sided at the ends, normalised; the
// binormal normalize(t_i x n_i) (b_0 from tangent_frame); the arclength a warp scan of the
// segment lengths.  Lanes past the strand's end return zeros.
__device__ __forceinline__ FramePoint frame_chunk(const float* p, int V, int c0, int lane, FrameCarry& cy) {
    const int i = c0 + lane;
    const bool valid = i < V;
    const V3 z = v3(0.f, 0.f, 0.f);
    const V3 pi = valid ? ld3(p + 3 * i) : z;
    V3 pn = shfl_down3(pi, 1), pp = shfl_up3(pi, 1);
    if (lane == 31 && i + 1 < V) pn = ld3(p + 3 * (i + 1));
    if (lane == 0) pp = cy.p_last;
    V3 t = z;
    if (valid) {
        if (i + 1 < V) t = add(t, sub(pn, pi));
        if (i > 0) t = add(t, sub(pi, pp));
        t = unit(t);
    }
    V3 tp = shfl_up3(t, 1);
    if (lane == 0) tp = cy.t_last;
    M3 P = m3_identity();
    float arc = 0.f;
    if (valid && i > 0) {
        const V3 v1 = sub(pi, pp);
        const float c1 = fmaxf(dot(v1, v1), 1e-8f);
        const M3 H1 = householder(v1, 2.f / c1);
        const V3 v2 = sub(t, m3_vec(H1, tp));
        const float c2 = fmaxf(dot(v2, v2), 1e-8f);
        P = m3_mul(householder(v2, 2.f / c2), H1);
        arc = norm(v1);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        M3 Q;
#pragma unroll
        for (int k = 0; k < 9; ++k) Q.m[k] = __shfl_up_sync(0xffffffffu, P.m[k], d);
        const float ua = __shfl_up_sync(0xffffffffu, arc, d);
        if (lane >= d) {
            P = m3_mul(P, Q);
            arc += ua;
        }
    }
    arc += cy.arc;
    V3 n = cy.n0, b = cy.b0;
    if (i > 0) {
        n = unit(m3_vec(P, cy.n_prev));
        b = unit(cross(t, n));
    }
    if (!valid) {
        n = z;
        b = z;
    }
    cy.n_prev = shfl3(n, 31);
    cy.arc = shfl_f(arc, 31);
    cy.p_last = shfl3(pi, 31);
    cy.t_last = shfl3(t, 31);
    return FramePoint{pi, t, n, b, arc};
}

// [t_dst n_dst b_dst] [t n b]^T, row-major
__device__ __forceinline__ void align_rotation(V3 td, V3 nd, V3 bd, V3 t, V3 n, V3 b, float R[9]) {
    const float dc[3][3] = {{td.x, nd.x, bd.x}, {td.y, nd.y, bd.y}, {td.z, nd.z, bd.z}};
    const float sc[3][3] = {{t.x, n.x, b.x}, {t.y, n.y, b.y}, {t.z, n.z, b.z}};
#pragma unroll
    for (int rr = 0; rr < 3; ++rr)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            R[3 * rr + cc] = (dc[rr][0] * sc[cc][0] + dc[rr][1] * sc[cc][1]) + dc[rr][2] * sc[cc][2];
}

// compute_bishop_frame (curve_utils.py:104-165) + compute_alignment_rotation (:273-308) +
// compute_aligned_strands (:243-271): one warp per strand, one lane per point (frame_chunk);
// each warp writes its 32 points' outputs through shared memory as contiguous runs.
__global__ void __launch_bounds__(kFrameThreads, 4) strand_frames_kernel(FrameArgs a) {
    __shared__ float sbuf[kFrameWarps][32 * 9];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* wbuf = sbuf[warp];
    const int V = a.V;
    const V3 td = a.tdst;
    const int64_t nwarps = (int64_t)gridDim.x * kFrameWarps;
    for (int64_t s = (int64_t)blockIdx.x * kFrameWarps + warp; s < a.N; s += nwarps) {
        const float* p = a.strands + s * V * 3;
        FrameCarry cy;
        frame_root(p, V, td, a.R != nullptr, cy);
        const V3 root = a.roots ? ld3(a.roots + a.roots_stride * s) : ld3(p);
        for (int c0 = 0; c0 < V; c0 += 32) {
            const FramePoint f = frame_chunk(p, V, c0, lane, cy);
            const int nitems = min(32, V - c0);
            const int64_t o = s * V + c0;
            if (a.T) warp_store<3>(wbuf, {f.t.x, f.t.y, f.t.z}, a.T + 3 * o, nitems, lane);
            if (a.Nn) warp_store<3>(wbuf, {f.n.x, f.n.y, f.n.z}, a.Nn + 3 * o, nitems, lane);
            if (a.Bn) warp_store<3>(wbuf, {f.b.x, f.b.y, f.b.z}, a.Bn + 3 * o, nitems, lane);
            if (a.R) {
                float R[9];
                align_rotation(td, cy.nd, cy.bd, f.t, f.n, f.b, R);
                warp_store<9>(wbuf, R, a.R + 9 * o, nitems, lane);
            }
            if (a.canon) {
                const V3 cn = add(mul(td, f.arc), root);
                warp_store<3>(wbuf, {cn.x, cn.y, cn.z}, a.canon + 3 * o, nitems, lane);
            }
        }
    }
}

// Eigenvectors of a symmetric 3x3 (cyclic Jacobi, FP32): columns of E, eigenvalues in w.
// Each rotation zeroes its (p, q) entry exactly; an entry below 1e-9 of its diagonal pair
// counts as zero, so the sweeps stop once all three off-diagonal entries are zero (a few
// sweeps; at most 16).  FP32 on purpose: this GPU's FP64 rate is a small fraction of its
// FP32 rate, and the least-variance axis the frame needs is resolved to about
// eps * lambda_max / (lambda_mid - lambda_min) either way.
template <int P, int Q>
__device__ __forceinline__ void jacobi_rotate(float (&A)[3][3], float (&E)[3][3]) {
    constexpr int R = 3 - P - Q;   // the third index
    const float apq = A[P][Q];
    if (apq == 0.f) return;
    if (fabsf(apq) <= 1e-9f * (fabsf(A[P][P]) + fabsf(A[Q][Q]))) {
        A[P][Q] = A[Q][P] = 0.f;
        return;
    }
    const float th = (A[Q][Q] - A[P][P]) / (2.f * apq);
    const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(th * th + 1.f));
    const float c = 1.f / sqrtf(t * t + 1.f), s = t * c;
    // J^T A J with J the rotation in the (P, Q) plane
    const float app = A[P][P], aqq = A[Q][Q], arp = A[R][P], arq = A[R][Q];
    A[P][P] = app - t * apq;
    A[Q][Q] = aqq + t * apq;
    A[P][Q] = A[Q][P] = 0.f;
    A[R][P] = A[P][R] = c * arp - s * arq;
    A[R][Q] = A[Q][R] = s * arp + c * arq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ekp = E[k][P], ekq = E[k][Q];
        E[k][P] = c * ekp - s * ekq;
        E[k][Q] = s * ekp + c * ekq;
    }
}

__device__ void jacobi3(float (&A)[3][3], float (&E)[3][3], float (&w)[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) E[i][j] = i == j ? 1.f : 0.f;
    for (int sweep = 0; sweep < 16; ++sweep) {
        if (A[0][1] == 0.f && A[0][2] == 0.f && A[1][2] == 0.f) break;
        jacobi_rotate<0, 1>(A, E);
        jacobi_rotate<0, 2>(A, E);
        jacobi_rotate<1, 2>(A, E);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// compensated running sum (Kahan)
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

constexpr int kWispThreads = 256;
constexpr int kWispWarps = kWispThreads / 32;

// Per wisp (align_wisps, curve_utils.py:521-568): root centre, longest strand, least-variance
// axis of the centred roots, and R_global = R_dst R_src^T with the reference's frames.
// A warp per strand sums the segment lengths (lanes over segments, coalesced) and lane 0
// keeps a compensated sum of the roots; the centred second moment is summed per thread and
// reduced in a tree; thread 0 solves the 3x3 eigenproblem and builds the frame.
__global__ void __launch_bounds__(kWispThreads) wisp_frames_kernel(int num_wisps, const int32_t* __restrict__ offs,
                                                                   int64_t num_strands, int V,
                                                                   const float* __restrict__ strands, V3 tdst,
                                                                   V3 ndst, V3 bdst, float* __restrict__ Rg,
                                                                   float* __restrict__ centre,
                                                                   int32_t* __restrict__ longest) {
    __shared__ float red[6][kWispWarps];
    __shared__ float wlen[kWispWarps];
    __shared__ int widx[kWispWarps];
    __shared__ float cen[3];
    const int w = blockIdx.x;
    if (w >= num_wisps) return;
    const int s0 = offs[w], s1 = offs[w + 1], n = s1 - s0;
    if (s0 < 0 || n <= 0 || (int64_t)s1 > num_strands) {
        // an empty or out-of-range wisp: identity frame, no guide
        if (threadIdx.x < 9) Rg[9 * w + threadIdx.x] = (threadIdx.x % 4 == 0) ? 1.f : 0.f;
        if (threadIdx.x < 3) centre[3 * w + threadIdx.x] = 0.f;
        if (threadIdx.x == 0) longest[w] = -1;
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // lengths (a warp per strand) and the root sum
    KSum sx, sy, sz;
    float best = -1.f;
    int bidx = 0x7fffffff;
    for (int s = s0 + warp; s < s1; s += kWispWarps) {
        const float* p = strands + (int64_t)s * V * 3;
        float len = 0.f;
        for (int i = 1 + lane; i < V; i += 32) len += norm(sub(ld3(p + 3 * i), ld3(p + 3 * (i - 1))));
        len = warp_sum_f(len);
        if (lane == 0) {
            sx.add(p[0]);
            sy.add(p[1]);
            sz.add(p[2]);
            if (len > best) {   // strands come in increasing order: the first of equal lengths stays
                best = len;
                bidx = s;
            }
        }
    }
    if (lane == 0) {
        red[0][warp] = sx.s;
        red[1][warp] = sy.s;
        red[2][warp] = sz.s;
        red[3][warp] = sx.c;
        red[4][warp] = sy.c;
        red[5][warp] = sz.c;
        wlen[warp] = best;
        widx[warp] = bidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        KSum tx, ty, tz;
        float bl = -1.f;
        int bi = 0x7fffffff;
        for (int k = 0; k < kWispWarps; ++k) {
            tx.add(red[0][k]);
            tx.add(-red[3][k]);
            ty.add(red[1][k]);
            ty.add(-red[4][k]);
            tz.add(red[2][k]);
            tz.add(-red[5][k]);
            if (wlen[k] > bl || (wlen[k] == bl && widx[k] < bi)) {
                bl = wlen[k];
                bi = widx[k];
            }
        }
        cen[0] = tx.s / (float)n;
        cen[1] = ty.s / (float)n;
        cen[2] = tz.s / (float)n;
        widx[0] = bi;
    }
    __syncthreads();
    const V3 c = v3(cen[0], cen[1], cen[2]);
    const int gsel = widx[0];
    // second moment of the centred roots
    float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int s = s0 + threadIdx.x; s < s1; s += kWispThreads) {
        const V3 x = sub(ld3(strands + (int64_t)s * V * 3), c);
        m[0] += x.x * x.x;
        m[1] += x.x * x.y;
        m[2] += x.x * x.z;
        m[3] += x.y * x.y;
        m[4] += x.y * x.z;
        m[5] += x.z * x.z;
    }
    __syncthreads();   // every thread has read cen and widx[0] before red is reused
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        m[k] = warp_sum_f(m[k]);
        if (lane == 0) red[k][warp] = m[k];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    float M[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        float a = 0.f;
        for (int j = 0; j < kWispWarps; ++j) a += red[k][j];
        M[k] = a;
    }
    V3 least = v3(0.f, 0.f, 1.f), second = v3(0.f, 1.f, 0.f);
    if (n >= 3) {
        float A[3][3] = {{M[0], M[1], M[2]}, {M[1], M[3], M[4]}, {M[2], M[4], M[5]}};
        float E[3][3], ev[3];
        jacobi3(A, E, ev);
        // descending eigenvalue (singular value) order: principal, second, least
        const int i_max = (ev[0] >= ev[1] && ev[0] >= ev[2]) ? 0 : (ev[1] >= ev[2] ? 1 : 2);
        const int i_min = (ev[2] <= ev[1] && ev[2] <= ev[0] && i_max != 2) ? 2
                          : ((ev[1] <= ev[0] && i_max != 1) ? 1 : (i_max != 0 ? 0 : 1));
        const int i_mid = 3 - i_max - i_min;
        least = v3(i_min == 0 ? E[0][0] : i_min == 1 ? E[0][1] : E[0][2],
                   i_min == 0 ? E[1][0] : i_min == 1 ? E[1][1] : E[1][2],
                   i_min == 0 ? E[2][0] : i_min == 1 ? E[2][1] : E[2][2]);
        second = v3(i_mid == 0 ? E[0][0] : i_mid == 1 ? E[0][1] : E[0][2],
                    i_mid == 0 ? E[1][0] : i_mid == 1 ? E[1][1] : E[1][2],
                    i_mid == 0 ? E[2][0] : i_mid == 1 ? E[2][1] : E[2][2]);
    }
    const int gi = (gsel >= s0 && gsel < s1) ? gsel : s0;   // all lengths NaN: the first strand
    longest[w] = gi;
    const float* g = strands + (int64_t)gi * V * 3;
    const V3 g0 = sub(ld3(g), c), g1 = sub(ld3(g + 3), c), gl = sub(ld3(g + 3 * (V - 1)), c);
    const V3 view = unit(sub(g0, g1)), down = unit(sub(gl, g0));
    const float sg = dot(least, view);
    const V3 nsrc = mul(least, sg < 0.f ? -1.f : 1.f);
    V3 tsrc = sub(down, mul(nsrc, dot(down, nsrc)));
    tsrc = mul(tsrc, 1.f / norm(tsrc));
    if (!(isfinite(tsrc.x) && isfinite(tsrc.y) && isfinite(tsrc.z))) tsrc = second;
    const V3 bsrc = cross(tsrc, nsrc);
    const float dc[3][3] = {{tdst.x, ndst.x, bdst.x}, {tdst.y, ndst.y, bdst.y}, {tdst.z, ndst.z, bdst.z}};
    const float sc[3][3] = {{tsrc.x, nsrc.x, bsrc.x}, {tsrc.y, nsrc.y, bsrc.y}, {tsrc.z, nsrc.z, bsrc.z}};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
            Rg[9 * w + 3 * r + cc] = (dc[r][0] * sc[cc][0] + dc[r][1] * sc[cc][1]) + dc[r][2] * sc[cc][2];
    st3(centre + 3 * w, c);
}

// R (x - c), the expression both wisp_rotate_kernel and align_strands_kernel use
__device__ __forceinline__ V3 rotate_about(const float R[9], V3 c, V3 x) {
    x = sub(x, c);
    return v3((R[0] * x.x + R[1] * x.y) + R[2] * x.z, (R[3] * x.x + R[4] * x.y) + R[5] * x.z,
              (R[6] * x.x + R[7] * x.y) + R[8] * x.z);
}

// the wisp holding strand s (binary search over the offsets by lane 0, broadcast), or -1;
// R, c receive its frame (identity and 0 for no wisp)
__device__ __forceinline__ int wisp_of_strand(int64_t s, int num_wisps, const int32_t* __restrict__ offs,
                                              const float* __restrict__ Rg, const float* __restrict__ centre,
                                              int lane, float R[9], V3& c) {
    int w = -1;
    if (lane == 0 && num_wisps > 0 && s >= offs[0] && s < offs[num_wisps]) {
        int lo = 0, hi = num_wisps - 1;   // last w with offs[w] <= s
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (offs[mid] <= s) lo = mid; else hi = mid - 1;
        }
        if (offs[lo] <= s && s < offs[lo + 1]) w = lo;
    }
    w = __shfl_sync(0xffffffffu, w, 0);
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.f : 0.f;
    c = v3(0.f, 0.f, 0.f);
    if (w >= 0) {
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = __ldg(Rg + 9 * w + k);
        c = ld3(centre + 3 * w);
    }
    return w;
}

// a_out = R_w (a - centre_w) and b_out likewise for every point of every strand, w the wisp
// whose offsets range holds the strand (a strand of no wisp is copied unchanged): a warp per
// strand, lanes over the points.
__global__ void __launch_bounds__(256) wisp_rotate_kernel(int64_t num_strands, int V, int num_wisps,
                                                          const int32_t* __restrict__ offs,
                                                          const float* __restrict__ Rg,
                                                          const float* __restrict__ centre,
                                                          const float* __restrict__ a, const float* __restrict__ b,
                                                          float* __restrict__ ao, float* __restrict__ bo) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < num_strands; s += nw) {
        float R[9];
        V3 c;
        const int w = wisp_of_strand(s, num_wisps, offs, Rg, centre, lane, R, c);
        const int64_t o = s * V;
        for (int i = lane; i < V; i += 32) {
            const V3 x = ld3(a + 3 * (o + i)), y = ld3(b + 3 * (o + i));
            st3(ao + 3 * (o + i), w >= 0 ? rotate_about(R, c, x) : x);
            st3(bo + 3 * (o + i), w >= 0 ? rotate_about(R, c, y) : y);
        }
    }
}

// align_wisps after the per-wisp frames (curve_utils.py:487-606), one warp per strand with the
// strand staged in shared memory: smoothing (the handle strand, written out), rotation of
// the strand and its handle into the wisp frame, rotation-minimising frames of the rotated
// handle (frame_chunk) with its alignment rotations and canonical handles, and skinning of
// the rotated strand.  The same device code as smooth_strands, wisp_rotate, strand_frames
// and skinning, in the same order, so the result equals that composition bit for bit while
// only the strands are read and the handles and aligned strands written.
constexpr int kAlignFloatsPerPoint = 19;   // x 3, handle 3, R 9, canonical 3, arclength 1
constexpr int kAlignSmemMax = 96 * 1024;

struct AlignArgs {
    int64_t N;
    int V;
    const float* strands;
    int num_wisps;
    const int32_t* offs;
    const float* Rg;
    const float* centre;
    V3 td;
    float beta;
    float* handles;   // (N, V, 3): the smoothed strands before alignment
    float* aligned;   // (N, V, 3)
};

__global__ void __launch_bounds__(256, 4) align_strands_kernel(AlignArgs a) {
    extern __shared__ float asm_[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps_cta = blockDim.x >> 5;
    const int V = a.V;
    float* sx = asm_ + (size_t)warp * kAlignFloatsPerPoint * V;
    float* sh = sx + 3 * V;
    float* sR = sh + 3 * V;
    float* sc = sR + 9 * V;
    float* sarc = sc + 3 * V;
    const float inv_beta2 = __fdiv_rn(1.0f, __fmul_rn(a.beta, a.beta));
    const float cutoff = __fmul_rn(3.0f, a.beta);
    const int64_t nw = (int64_t)gridDim.x * nwarps_cta;
    for (int64_t s = (int64_t)blockIdx.x * nwarps_cta + warp; s < a.N; s += nw) {
        float R[9];
        V3 c;
        const int w = wisp_of_strand(s, a.num_wisps, a.offs, a.Rg, a.centre, lane, R, c);
        const int64_t o = s * V;
        for (int k = lane; k < 3 * V; k += 32) sx[k] = __ldg(a.strands + 3 * o + k);
        __syncwarp();
        warp_arclength(sx, V, sarc, lane);
        __syncwarp();
        // the handle strand: smoothed, written out, rotated into the wisp frame
        for (int i = lane; i < V; i += 32) {
            float h3[3];
            smooth_point(sx, sarc, V, i, cutoff, inv_beta2, true, h3);
            const V3 h = v3(h3[0], h3[1], h3[2]);
            st3(a.handles + 3 * (o + i), h);
            st3(sh + 3 * i, w >= 0 ? rotate_about(R, c, h) : h);
        }
        __syncwarp();
        for (int i = lane; i < V; i += 32) {
            const V3 x = ld3(sx + 3 * i);
            st3(sx + 3 * i, w >= 0 ? rotate_about(R, c, x) : x);
        }
        __syncwarp();
        // frames of the rotated handle: rotations and canonical handles
        FrameCarry cy;
        frame_root(sh, V, a.td, true, cy);
        const V3 root = ld3(sx);
        for (int c0 = 0; c0 < V; c0 += 32) {
            const FramePoint f = frame_chunk(sh, V, c0, lane, cy);
            const int i = c0 + lane;
            if (i < V) {
                align_rotation(a.td, cy.nd, cy.bd, f.t, f.n, f.b, sR + 9 * i);
                st3(sc + 3 * i, add(mul(a.td, f.arc), root));
            }
        }
        __syncwarp();
        warp_arclength(sx, V, sarc, lane);
        __syncwarp();
        for (int i = lane; i < V; i += 32) {
            float o3[3];
            skin_point(sx, sarc, sh, sc, sR, V, i, cutoff, inv_beta2, true, o3);
            st3(a.aligned + 3 * (o + i), v3(o3[0], o3[1], o3[2]));
        }
        __syncwarp();
    }
}

}  // namespace
}  // namespace s2c

using namespace s2c;

extern "C" S2C_API s2c_status s2c_strand_frames(int N, int V, const float* strands, const float* t_dst, float* T,
                                                float* Nrm, float* Bin, float* R, const float* roots,
                                                int64_t roots_stride, float* canon, s2c_stream stream) {
    S2C_REQUIRE(N >= 0 && V >= 0, "strand_frames: bad sizes");
    if (N == 0 || V == 0) return S2C_OK;
    S2C_REQUIRE(strands, "strand_frames: null strands");
    S2C_REQUIRE((!R && !canon) || t_dst, "strand_frames: rotations and canonical handles need t_dst");
    S2C_REQUIRE(!roots || roots_stride >= 3, "strand_frames: roots stride below 3");
    FrameArgs a;
    a.N = N;
    a.V = V;
    a.strands = strands;
    a.tdst = t_dst ? v3(t_dst[0], t_dst[1], t_dst[2]) : v3(0.f, 1.f, 0.f);
    a.T = T;
    a.Nn = Nrm;
    a.Bn = Bin;
    a.R = R;
    a.roots = roots;
    a.roots_stride = roots_stride;
    a.canon = canon;
    strand_frames_kernel<<<grid_for(N, kFrameWarps, (int64_t)num_sms() * 8), kFrameThreads, 0,
                           (cudaStream_t)stream>>>(a);
    S2C_CHECK_LAUNCH("strand_frames_kernel");
    return S2C_OK;
}

extern "C" S2C_API s2c_status s2c_wisp_frames(int num_wisps, const int32_t* offsets, int64_t num_strands, int V,
                                              const float* strands,
                                              const float* t_dst, const float* n_dst, const float* b_dst,
                                              float* R_global, float* centre, int32_t* longest, s2c_stream stream) {
    S2C_REQUIRE(num_wisps >= 0 && V >= 2, "wisp_frames: bad sizes");
    if (num_wisps == 0) return S2C_OK;
    S2C_REQUIRE(offsets && strands && t_dst && n_dst && b_dst && R_global && centre && longest,
                "wisp_frames: null pointer");
    wisp_frames_kernel<<<num_wisps, 256, 0, (cudaStream_t)stream>>>(
        num_wisps, offsets, num_strands, V, strands, v3(t_dst[0], t_dst[1], t_dst[2]), v3(n_dst[0], n_dst[1], n_dst[2]),
        v3(b_dst[0], b_dst[1], b_dst[2]), R_global, centre, longest);
    S2C_CHECK_LAUNCH("wisp_frames_kernel");
    return S2C_OK;
}

extern "C" S2C_API s2c_status s2c_wisp_rotate(int num_wisps, const int32_t* offsets, int64_t num_strands, int V,
                                              const float* R_global, const float* centre, const float* a,
                                              const float* b, float* a_out, float* b_out, s2c_stream stream) {
    S2C_REQUIRE(num_wisps >= 0 && num_strands >= 0 && V > 0, "wisp_rotate: bad sizes");
    if (num_strands == 0) return S2C_OK;
    S2C_REQUIRE(a && b && a_out && b_out && (num_wisps == 0 || (offsets && R_global && centre)),
                "wisp_rotate: null pointer");
    wisp_rotate_kernel<<<grid_for(num_strands, 8, (int64_t)num_sms() * 16), 256, 0, (cudaStream_t)stream>>>(
        num_strands, V, num_wisps, offsets, R_global, centre, a, b, a_out, b_out);
    S2C_CHECK_LAUNCH("wisp_rotate_kernel");
    return S2C_OK;
}

extern "C" S2C_API int s2c_align_strands_max_points(void) {
    return kAlignSmemMax / (kAlignFloatsPerPoint * 4);
}

extern "C" S2C_API s2c_status s2c_align_strands(int64_t num_strands, int V, const float* strands, int num_wisps,
                                                const int32_t* offsets, const float* R_global, const float* centre,
                                                const float* t_dst, float beta, float* handles, float* aligned,
                                                s2c_stream stream) {
    S2C_REQUIRE(num_strands >= 0 && num_wisps >= 0 && V >= 2, "align_strands: bad sizes");
    S2C_REQUIRE(V <= s2c_align_strands_max_points(), "align_strands: strands of %d points exceed the staged limit of %d",
                V, s2c_align_strands_max_points());
    if (num_strands == 0) return S2C_OK;
    S2C_REQUIRE(strands && t_dst && handles && aligned && (num_wisps == 0 || (offsets && R_global && centre)),
                "align_strands: null pointer");
    AlignArgs a;
    a.N = num_strands;
    a.V = V;
    a.strands = strands;
    a.num_wisps = num_wisps;
    a.offs = offsets;
    a.Rg = R_global;
    a.centre = centre;
    a.td = v3(t_dst[0], t_dst[1], t_dst[2]);
    a.beta = beta;
    a.handles = handles;
    a.aligned = aligned;
    const size_t per_warp = (size_t)kAlignFloatsPerPoint * 4 * V;
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, kAlignSmemMax / per_warp));
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024)   // per call: the attribute belongs to the current device
        cudaFuncSetAttribute(align_strands_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int per_sm = std::max(1, (int)(200 * 1024 / smem));
    align_strands_kernel<<<grid_for(num_strands, warps, (int64_t)num_sms() * per_sm), warps * 32, smem,
                           (cudaStream_t)stream>>>(a);
    S2C_CHECK_LAUNCH("align_strands_kernel");
    return S2C_OK;
}
