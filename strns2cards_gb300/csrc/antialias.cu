// Silhouette edges and the antialiased-bitset edge gradient (the reference's antialias.cu).
//
// mark: one thread per (view, edge), the reference's FP32 arithmetic (the projection
//   multiply of the second vertex is fused into each coordinate difference, as the
//   reference build does), so silhouette decisions and normals are bit-identical.
// backward: one warp per silhouette fragment.  The reference's thread walks the 15 x 15
//   Gaussian window serially with two scattered bitset reads per tap; here the 32 lanes
//   take the taps together (32 independent reads in flight), reduce with shuffles, and
//   lane 0 applies the chain rule.  Decisions (half-pixel test, disk cutoff) are FP32 as in
//   the reference; the weights use expf and the window sum is accumulated in FP64.
#include <algorithm>

#include "aa.cuh"
#include "common.cuh"
#include "scan.cuh"

namespace s2c {

struct Mesh {
    const float4* __restrict__ pos4;  // (B, V)
    const int* __restrict__ tri;      // (T, 3)
    const int2* __restrict__ edges;   // (E)
    const int2* __restrict__ e2t;     // (E)
    int V, T, E;
    FastDiv divE;
};

// mark_edge_t for edge e of view b of a mesh in global memory
struct GlobalPos {
    const float4* __restrict__ p;
    __device__ __forceinline__ float4 operator()(int v) const { return __ldg(p + v); }
};

__device__ __forceinline__ int mark_edge(int H, int W, const Mesh& M, int b, int e, float2& nrm) {
    return mark_edge_t(H, W, __ldg(M.edges + e), __ldg(M.e2t + e), M.tri, M.T, M.V, GlobalPos{M.pos4 + (int64_t)b * M.V},
                       nrm);
}

__global__ void __launch_bounds__(256) mark_edges_kernel(int H, int W, int B, Mesh M, int32_t* __restrict__ prim_ids,
                                                         float2* __restrict__ normals) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * M.E) return;
    const int b = (int)M.divE.div((uint32_t)idx);
    const int e = (int)idx - b * M.E;
    float2 nrm;
    const int m = mark_edge(H, W, M, b, e, nrm);
    if (m == 2) prim_ids[idx] = (int32_t)idx;
    if (m >= 1) normals[idx] = nrm;
}

struct AAArgs {
    int64_t F;
    const int32_t* __restrict__ frag_pix;
    const float4* __restrict__ frag_attrs;
    int B, H, W, S;
    const int32_t* __restrict__ bitset;
    const int32_t* __restrict__ target;
    const float4* __restrict__ pos4;
    int V, E;
    const int2* __restrict__ edges;
    const float2* __restrict__ normals;
    const int32_t* __restrict__ e2c;
    float* __restrict__ d_pos;
    double* __restrict__ acc64;     // non-null: contributions summed in FP64 here instead
    const uint32_t* __restrict__ pplanes;  // cluster planes of bitset / target (B, 32 S, H, WQ)
    const uint32_t* __restrict__ tplanes;
    int WQ;
    float kr, rho;
};

__device__ __forceinline__ int plane_bit(const uint32_t* __restrict__ planes, const AAArgs& A, int b, int c, int y,
                                         int x) {
    return (__ldg(planes + (((int64_t)b * 32 * A.S + c) * A.H + y) * A.WQ + (x >> 5)) >> (x & 31)) & 1;
}

__device__ __forceinline__ int bit_of(const int32_t* __restrict__ bits, int64_t pix, int S, int c) {
    return (__ldg(bits + pix * S + (c >> 5)) >> (c & 31)) & 1;
}

// The window part of antialias.cu:121-279 for one fragment (view b, pixel (h, w), sweep
// axis, t1, edge e), evaluated by a whole warp: every lane computes the (uniform) set-up,
// the lanes share the taps, and the FP64 window sum is reduced over the warp.  Returns
// false when the fragment contributes nothing; otherwise dc (on every lane) and the
// quantities of the chain rule.
struct AAFrag {
    float dc;
    float px, py, pw, t0, t1;
    float2 nrm;
    int2 ev;
};

// Per-fragment set-up of antialias.cu:121-176 (edge point, half-pixel test, neighbour,
// c01 and the window bounds); false when the fragment contributes nothing.
struct AAPrep {
    float fx, fy, px, py, pw, t0, t1;
    float2 nrm;
    int2 ev;
    int c, c01, h0, h1, w0, w1;
};

template <bool kPlanes>
__device__ __forceinline__ bool aa_prep(const AAArgs& A, int b, int h, int w, float axis, float t1, int e, float2 nrm,
                                        AAPrep& P) {
    const float fH = (float)A.H, fW = (float)A.W;
    if (e < 0 || e >= A.E || b < 0 || b >= A.B || h < 0 || h >= A.H || w < 0 || w >= A.W) return false;
    const float t0 = __fsub_rn(1.f, t1);
    const int2 ev = __ldg(A.edges + e);
    if ((unsigned)ev.x >= (unsigned)A.V || (unsigned)ev.y >= (unsigned)A.V) return false;
    const float4 p0 = __ldg(A.pos4 + (int64_t)b * A.V + ev.x), p1 = __ldg(A.pos4 + (int64_t)b * A.V + ev.y);
    const float px = __fmaf_rn(t0, p0.x, __fmul_rn(t1, p1.x));
    const float py = __fmaf_rn(t0, p0.y, __fmul_rn(t1, p1.y));
    const float pw = __fmaf_rn(t0, p0.w, __fmul_rn(t1, p1.w));
    const float fx = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(1.f, __fdiv_rn(px, pw))), fW);
    const float fy = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, __fdiv_rn(py, pw))), fH);
    const float rx = __fsub_rn(fx, floorf(fx)), ry = __fsub_rn(fy, floorf(fy));
    int nh = h, nw = w;
    float dot;
    if (axis == 0.f) {
        if (!isfinite(rx) || fabsf(__fsub_rn(rx, 0.5f)) >= 1e-4f) return false;
        const int d = 2 * (int)(ry > 0.5f) - 1;
        nh += d;
        dot = __fmul_rn((float)d, nrm.y);
    } else {
        if (!isfinite(ry) || fabsf(__fsub_rn(ry, 0.5f)) >= 1e-4f) return false;
        const int d = 2 * (int)(rx > 0.5f) - 1;
        nw += d;
        dot = __fmul_rn((float)d, nrm.x);
    }
    if (nw < 0 || nw >= A.W || nh < 0 || nh >= A.H || dot == 0.f) return false;
    const int c = __ldg(A.e2c + e);
    if (c < 0 || c >= 32 * A.S) return false;
    const int64_t img = (int64_t)b * A.H * A.W;
    int c01;
    if (kPlanes)
        c01 = 1 - (dot > 0.f ? plane_bit(A.pplanes, A, b, c, nh, nw) : plane_bit(A.pplanes, A, b, c, h, w));
    else
        c01 = 1 - (dot > 0.f ? bit_of(A.bitset, img + (int64_t)nh * A.W + nw, A.S, c)
                             : bit_of(A.bitset, img + (int64_t)h * A.W + w, A.S, c));
    if (c01 == 0) return false;
    const int R = f2i(floorf(A.kr));
    const int cw = f2i(floorf(fx)), ch = f2i(floorf(fy));
    P.h0 = max(ch - R, 0);
    P.h1 = min(ch + R, A.H - 1) + 1;
    P.w0 = max(cw - R, 0);
    P.w1 = min(cw + R, A.W - 1) + 1;
    aa_trim_window(A.kr, fx, fy, P.h0, P.h1, P.w0, P.w1);
    P.fx = fx;
    P.fy = fy;
    P.px = px;
    P.py = py;
    P.pw = pw;
    P.t0 = t0;
    P.t1 = t1;
    P.nrm = nrm;
    P.ev = ev;
    P.c = c;
    P.c01 = c01;
    return true;
}

template <bool kPlanes>
__device__ __forceinline__ bool aa_fragment(const AAArgs& A, int b, int h, int w, float axis, float t1, int e,
                                            float2 nrm, int lane, AAFrag& o) {
    AAPrep P;
    if (!aa_prep<kPlanes>(A, b, h, w, axis, t1, e, nrm, P)) return false;
    const int h0 = P.h0, h1 = P.h1, w0 = P.w0, w1 = P.w1;
    const float fx = P.fx, fy = P.fy, px = P.px, py = P.py, pw = P.pw, t0 = P.t0;
    const int2 ev = P.ev;
    const int c = P.c, c01 = P.c01;
    const int64_t img = (int64_t)b * A.H * A.W;
    const int ww = w1 - w0, taps = ww > 0 && h1 > h0 ? ww * (h1 - h0) : 0;
    const AAWin q = aa_win(A.kr);
    const float cc = q.cc, alpha = q.alpha, kr2 = q.kr2;
    // each lane sums its taps (at most ceil(taps / 32) of them) in FP32; the lanes' partial
    // sums are reduced in FP64.  Tap j = lane + 32 i sits at (row, col) = divmod(j, ww),
    // stepped incrementally.
    if (kPlanes) {
        // lanes take window rows; a row is read as the 1-2 plane words covering [w0, w1) of
        // both images, and only the pixels where they differ are visited, in x order
        float sum = 0.f, comp = 0.f;
        const int rows = taps > 0 ? h1 - h0 : 0;
        const int64_t pbase = ((int64_t)b * 32 * A.S + c) * A.H;
        for (int r = lane; r < rows; r += 32) {
            const int th = h0 + r;
            const uint32_t* prow = A.pplanes + (pbase + th) * A.WQ;
            const uint32_t* trow = A.tplanes + (pbase + th) * A.WQ;
            const float dy = __fsub_rn(__fadd_rn((float)th, 0.5f), fy);
            for (int q = w0 >> 5; q <= (w1 - 1) >> 5; ++q) {
                const int lo = max(w0 - 32 * q, 0), hi = min(w1 - 32 * q, 32);
                const uint32_t m = (hi == 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
                const uint32_t pv = __ldg(prow + q), tv = __ldg(trow + q);
                const uint32_t pos = pv & ~tv & m, neg = ~pv & tv & m;
                uint32_t any = pos | neg;
                while (any) {
                    const int bit = __ffs(any) - 1;
                    any &= any - 1;
                    const int tw = 32 * q + bit;
                    const float dx = __fsub_rn(__fadd_rn((float)tw, 0.5f), fx);
                    const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
                    if (!(n2 < kr2)) continue;
                    const float wgt = __fmul_rn(cc, expf(-alpha * n2));
                    kahan_add(sum, comp, ((pos >> bit) & 1u) ? __fmul_rn(wgt, A.rho) : -wgt);
                }
            }
        }
        o.dc = __fmul_rn((float)c01, warp_sum_comp(sum, comp));
        if (o.dc == 0.f) return false;
        o.px = px;
        o.py = py;
        o.pw = pw;
        o.t0 = t0;
        o.t1 = t1;
        o.nrm = nrm;
        o.ev = ev;
        return true;
    }
    float sum = 0.f, comp = 0.f;
    if (taps > 0) {
        const int s_row = 32 / ww, s_col = 32 - s_row * ww;
        int row = lane / ww, col = lane - (lane / ww) * ww;
        const int slot = c >> 5, bit = c & 31;
        for (int j = lane; j < taps; j += 32) {
            const int th = h0 + row, tw = w0 + col;
            const int64_t pix = (img + (int64_t)th * A.W + tw) * A.S + slot;
            const int c0 = (__ldg(A.bitset + pix) >> bit) & 1, c1 = (__ldg(A.target + pix) >> bit) & 1;
            row += s_row;
            col += s_col;
            if (col >= ww) {
                col -= ww;
                ++row;
            }
            if (c0 == c1) continue;
            const float dx = __fsub_rn(__fadd_rn((float)tw, 0.5f), fx);
            const float dy = __fsub_rn(__fadd_rn((float)th, 0.5f), fy);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < kr2)) continue;
            const float wgt = __fmul_rn(cc, expf(-alpha * n2));
            kahan_add(sum, comp, c0 ? __fmul_rn(wgt, A.rho) : -wgt);   // (c0 - c1) * (c1 == 0 ? rho : 1)
        }
    }
    o.dc = __fmul_rn((float)c01, warp_sum_comp(sum, comp));
    if (o.dc == 0.f) return false;
    o.px = px;
    o.py = py;
    o.pw = pw;
    o.t0 = t0;
    o.t1 = t1;
    o.nrm = nrm;
    o.ev = ev;
    return true;
}

// Chain rule of one fragment (antialias.cu:281-316)
__device__ __forceinline__ bool aa_chain(const AAArgs& A, const AAFrag& f, float& dpx, float& dpy, float& dpw) {
    return aa_chain_rule(A.H, A.W, f.dc, f.nrm, f.px, f.py, f.pw, dpx, dpy, dpw);
}

// antialias.cu:121-279, one warp per fragment of a fragment list
__global__ void __launch_bounds__(256) aa_backward_kernel(AAArgs A) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp0; i < A.F; i += nwarps) {
        const float4 fa = A.frag_attrs[i];
        const int fb = A.frag_pix[3 * i], fe = f2i(fa.w) - 1;
        if (fe < 0 || fe >= A.E || fb < 0 || fb >= A.B) continue;
        AAFrag f;
        if (!aa_fragment<false>(A, fb, A.frag_pix[3 * i + 1], A.frag_pix[3 * i + 2], fa.x, fa.y, fe,
                         __ldg(A.normals + (int64_t)fb * A.E + fe), lane, f))
            continue;
        if (lane != 0) continue;
        float dpx, dpy, dpw;
        if (!aa_chain(A, f, dpx, dpy, dpw)) continue;
        const int b = A.frag_pix[3 * i];
        if (A.acc64) {
            // contributions summed in FP64 at the L2 (no cancellation loss across fragments)
            double* a0 = A.acc64 + ((int64_t)b * A.V + f.ev.x) * 3;
            double* a1 = A.acc64 + ((int64_t)b * A.V + f.ev.y) * 3;
            atomicAdd(a0 + 0, (double)__fmul_rn(dpx, f.t0));
            atomicAdd(a0 + 1, (double)__fmul_rn(dpy, f.t0));
            atomicAdd(a0 + 2, (double)__fmul_rn(dpw, f.t0));
            atomicAdd(a1 + 0, (double)__fmul_rn(dpx, f.t1));
            atomicAdd(a1 + 1, (double)__fmul_rn(dpy, f.t1));
            atomicAdd(a1 + 2, (double)__fmul_rn(dpw, f.t1));
            continue;
        }
        // float atomics, as the reference
        float* g0 = A.d_pos + ((int64_t)b * A.V + f.ev.x) * 4;
        float* g1 = A.d_pos + ((int64_t)b * A.V + f.ev.y) * 4;
        atomicAdd(g0 + 0, __fmul_rn(dpx, f.t0));
        atomicAdd(g0 + 1, __fmul_rn(dpy, f.t0));
        atomicAdd(g0 + 3, __fmul_rn(dpw, f.t0));
        atomicAdd(g1 + 0, __fmul_rn(dpx, f.t1));
        atomicAdd(g1 + 1, __fmul_rn(dpy, f.t1));
        atomicAdd(g1 + 3, __fmul_rn(dpw, f.t1));
    }
}

// Fused edge gradient.  Pass 1 (thread per (view, edge)): the mark test and the DDA span
// count (the fragments dda_compute_fragments would list for the edge); a silhouette edge
// also leaves a record (end points, span, normal) for pass 2.  A device scan.  Pass 2
// (aa_frag_kernel): warps take equal chunks of the global fragment index space, 32
// fragments at a time:
//  1. each lane regenerates one fragment from its owner edge's record (the owner found by
//     a shuffle search over a 32-edge window of prefixes) with the DDA arithmetic --
//     coverage is recomputed, not stored -- and sets up its window (aa_prep);
//  2. the warp shares the window rows of its (up to 32) fragments: row i of the flattened
//     list goes to lane i % 32, which reads the 1-2 plane words of both images, visits the
//     pixels where they differ and leaves the row's compensated sum in shared memory.  A
//     thread per window would leave lanes idle while the warp's heaviest window finishes
//     (window work varies from nothing to the whole disk), and lanes whose fragment
//     contributes nothing would idle throughout;
//  3. each fragment's lane merges its rows' sums in row order (deterministic), applies the
//     chain rule and adds the contributions to the FP64 accumulator.
constexpr int kAAFragChunk = 64;
constexpr int kAARowCap = 256;    // row sums held per warp between merges

// a silhouette edge as pass 2 reads it
struct alignas(16) AAEdgeRec {
    float4 p0, p1;
    float sx, sy, slope, off0;
    float off1, axis;
    int count, b;
    float nx, ny;
    int e, pad;
};

// a fragment's window as the row-sharing lanes read it
struct AARowDesc {
    float fx, fy;
    int h0, first;      // first: the fragment's first row in the warp's flattened list
    int w0, w1;
    int64_t rowbase;    // word offset of row 0 of the fragment's cluster plane
};

__global__ void __launch_bounds__(256) aa_count_kernel(AAArgs A, Mesh M, int32_t* __restrict__ counts,
                                                       AAEdgeRec* __restrict__ recs) {
    const int64_t BE = (int64_t)A.B * M.E;
    for (int64_t pe = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pe < BE; pe += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)M.divE.div((uint32_t)pe);
        const int e = (int)pe - b * M.E;
        float2 nrm;
        int n = 0;
        if (mark_edge(A.H, A.W, M, b, e, nrm) == 2) {
            const int2 ev = __ldg(M.edges + e);
            const float4 p0 = __ldg(M.pos4 + (int64_t)b * M.V + ev.x), p1 = __ldg(M.pos4 + (int64_t)b * M.V + ev.y);
            const Span sp = dda_span(p0, p1, A.H, A.W);
            n = sp.count;
            if (n > 0) {
                AAEdgeRec r;
                r.p0 = p0;
                r.p1 = p1;
                r.sx = sp.sx;
                r.sy = sp.sy;
                r.slope = sp.slope;
                r.off0 = sp.off0;
                r.off1 = sp.off1;
                r.axis = sp.axis;
                r.count = sp.count;
                r.b = b;
                r.nx = nrm.x;
                r.ny = nrm.y;
                r.e = e;
                r.pad = 0;
                recs[pe] = r;
            }
        }
        counts[pe] = n;
    }
}

// One window row of a fragment: the pixels of [w0, w1) where the two planes differ, each
// weighted by the Gaussian (antialias.cu:177-206), as a Kahan FP32 sum (sum - comp).
__device__ __forceinline__ float2 aa_window_row(const AAArgs& A, const AARowDesc& r, int th, const AAWin& q) {
    const uint32_t* prow = A.pplanes + r.rowbase + (int64_t)th * A.WQ;
    const uint32_t* trow = A.tplanes + r.rowbase + (int64_t)th * A.WQ;
    const float dy = __fsub_rn(__fadd_rn((float)th, 0.5f), r.fy);
    float sum = 0.f, comp = 0.f;
    const int q0 = r.w0 >> 5, width = r.w1 - r.w0;
    if (width <= 32) {
        // the row as one 32-bit mask from w0 (one or two plane words), so that a lane's
        // pixels are one flat loop rather than a loop per word
        const int sh = r.w0 & 31;
        uint64_t pv = __ldg(prow + q0), tv = __ldg(trow + q0);
        if (sh + width > 32) {
            pv |= (uint64_t)__ldg(prow + q0 + 1) << 32;
            tv |= (uint64_t)__ldg(trow + q0 + 1) << 32;
        }
        const uint32_t m = width == 32 ? 0xffffffffu : (1u << width) - 1u;
        const uint32_t pw = (uint32_t)(pv >> sh) & m, tw = (uint32_t)(tv >> sh) & m;
        const uint32_t pos = pw & ~tw;
        uint32_t any = pw ^ tw;
        while (any) {
            const int bit = __ffs(any) - 1;
            any &= any - 1;
            const float dx = __fsub_rn(__fadd_rn((float)(r.w0 + bit), 0.5f), r.fx);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < q.kr2)) continue;
            const float wgt = __fmul_rn(q.cc, expf(-q.alpha * n2));
            kahan_add(sum, comp, ((pos >> bit) & 1u) ? __fmul_rn(wgt, A.rho) : -wgt);
        }
        return make_float2(sum, -comp);
    }
    for (int qq = q0; qq <= (r.w1 - 1) >> 5; ++qq) {
        const int lo = max(r.w0 - 32 * qq, 0), hi = min(r.w1 - 32 * qq, 32);
        const uint32_t m = (hi == 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
        const uint32_t pv = __ldg(prow + qq), tv = __ldg(trow + qq);
        const uint32_t pos = pv & ~tv & m;
        uint32_t any = (pv ^ tv) & m;
        while (any) {
            const int bit = __ffs(any) - 1;
            any &= any - 1;
            const float dx = __fsub_rn(__fadd_rn((float)(32 * qq + bit), 0.5f), r.fx);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < q.kr2)) continue;
            const float wgt = __fmul_rn(q.cc, expf(-q.alpha * n2));
            kahan_add(sum, comp, ((pos >> bit) & 1u) ? __fmul_rn(wgt, A.rho) : -wgt);
        }
    }
    return make_float2(sum, -comp);
}

__global__ void __launch_bounds__(256, 4) aa_frag_kernel(AAArgs A, const AAEdgeRec* __restrict__ recs,
                                                      const uint32_t* __restrict__ prefix,
                                                      const int64_t* __restrict__ total) {
    __shared__ AARowDesc s_desc[256];
    __shared__ float2 s_rows[8 * kAARowCap];
    const int lane = threadIdx.x & 31;
    AARowDesc* dsc = s_desc + (threadIdx.x & ~31);
    float2* rows_sum = s_rows + (threadIdx.x >> 5) * kAARowCap;
    const int64_t BE = (int64_t)A.B * A.E;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t tot64 = *total;
    if (tot64 > 0xffffffffLL) return;   // limit: 2^32 - 1 silhouette fragments per call (header)
    const uint32_t tot = (uint32_t)tot64;
    const AAWin win = aa_win(A.kr);
    const int64_t nch = ((int64_t)tot + kAAFragChunk - 1) / kAAFragChunk;
    for (int64_t ch = warp0; ch < nch; ch += nwarps) {
        const uint32_t c0 = (uint32_t)(ch * kAAFragChunk);
        const uint32_t c1 = (uint32_t)min((int64_t)tot, (ch + 1) * kAAFragChunk);
        int64_t lo = 0, hi = BE;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (__ldg(prefix + mid) <= c0) lo = mid + 1;
            else hi = mid;
        }
        int64_t t0 = lo;
        uint32_t start = t0 > 0 ? __ldg(prefix + t0 - 1) : 0u;
        uint32_t pre = t0 + lane < BE ? __ldg(prefix + t0 + lane) : 0xffffffffu;
        uint32_t base = c0;
        while (base < c1) {
            for (;;) {
                const unsigned m = __ballot_sync(0xffffffffu, pre <= base);
                if (!m) break;
                const int adv = __popc(m);
                start = __shfl_sync(0xffffffffu, pre, adv - 1);
                t0 += adv;
                pre = t0 + lane < BE ? __ldg(prefix + t0 + lane) : 0xffffffffu;
            }
            const uint32_t wend = __shfl_sync(0xffffffffu, pre, 31);
            const uint32_t end = min(min(c1, base + 32u), wend);
            const uint32_t j = base + lane;
            int ow = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const uint32_t pv = __shfl_sync(0xffffffffu, pre, ow + step - 1);
                if (pv <= j) ow += step;
            }
            const uint32_t prev = __shfl_sync(0xffffffffu, pre, ow > 0 ? ow - 1 : 0);
            base = end;
            // 1. this lane's fragment: the owner edge's record (the owner, j < end, has a
            //    non-zero count and so a record from pass 1 of this call)
            AAPrep P;
            bool ok = false;
            int b = 0;
            if (j < end) {
                const AAEdgeRec g = recs[t0 + ow];
                b = g.b;
                Span sp;
                sp.sx = g.sx;
                sp.sy = g.sy;
                sp.slope = g.slope;
                sp.off0 = g.off0;
                sp.off1 = g.off1;
                sp.axis = g.axis;
                sp.count = g.count;
                const int k = (int)(j - (ow > 0 ? prev : start));
                if (g.e >= 0 && k < sp.count) {
                    float x, y;
                    dda_sample(sp, k, x, y);
                    const int h = f2i(floorf(y)), w = f2i(floorf(x));
                    if (h >= 0 && h < A.H && w >= 0 && w < A.W) {
                        const float t1 = dda_t1(g.p0, g.p1, x, y, sp.axis, A.H, A.W);
                        if (z_ok(dda_z(g.p0, g.p1, t1)))
                            ok = aa_prep<true>(A, b, h, w, sp.axis, t1, prim_roundtrip(g.e), make_float2(g.nx, g.ny),
                                               P);
                    }
                }
            }
            // 2. the warp's window rows, flattened: fragment f owns rows [first_f, last_f)
            const int nrows = ok && P.w1 > P.w0 ? P.h1 - P.h0 : 0;
            int last = nrows;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, last, d);
                if (lane >= d) last += v;
            }
            const int all = __shfl_sync(0xffffffffu, last, 31);
            const int first = last - nrows;
            if (nrows) {
                AARowDesc r;
                r.fx = P.fx;
                r.fy = P.fy;
                r.h0 = P.h0;
                r.first = first;
                r.w0 = P.w0;
                r.w1 = P.w1;
                r.rowbase = ((int64_t)b * 32 * A.S + P.c) * A.H * A.WQ;
                dsc[lane] = r;
            }
            __syncwarp();
            float shi = 0.f, slo = 0.f;
            for (int r0 = 0; r0 < all; r0 += kAARowCap) {
                const int r1 = min(all, r0 + kAARowCap);
                for (int i0 = r0; i0 < r1; i0 += 32) {
                    const int i = i0 + lane;
                    int o = 0;   // the fragment of row i: the first lane whose last > i
#pragma unroll
                    for (int step = 16; step; step >>= 1) {
                        const int v = __shfl_sync(0xffffffffu, last, o + step - 1);
                        if (v <= i) o += step;
                    }
                    if (i >= r1) continue;
                    const AARowDesc r = dsc[o];
                    rows_sum[i - r0] = aa_window_row(A, r, r.h0 + (i - r.first), win);
                }
                __syncwarp();
                // 3. this fragment's rows of the batch, in order
                for (int i = max(first, r0); i < min(last, r1); ++i) {
                    const float2 v = rows_sum[i - r0];
                    two_sum_merge(shi, slo, v.x, v.y);
                }
                __syncwarp();
            }
            if (!nrows) continue;
            const float dc = __fmul_rn((float)P.c01, __fadd_rn(shi, slo));
            if (dc == 0.f) continue;
            float dpx, dpy, dpw;
            if (!aa_chain_rule(A.H, A.W, dc, P.nrm, P.px, P.py, P.pw, dpx, dpy, dpw)) continue;
            double* a0 = A.acc64 + ((int64_t)b * A.V + P.ev.x) * 3;
            double* a1 = A.acc64 + ((int64_t)b * A.V + P.ev.y) * 3;
            atomicAdd(a0 + 0, (double)__fmul_rn(dpx, P.t0));
            atomicAdd(a0 + 1, (double)__fmul_rn(dpy, P.t0));
            atomicAdd(a0 + 2, (double)__fmul_rn(dpw, P.t0));
            atomicAdd(a1 + 0, (double)__fmul_rn(dpx, P.t1));
            atomicAdd(a1 + 1, (double)__fmul_rn(dpy, P.t1));
            atomicAdd(a1 + 2, (double)__fmul_rn(dpw, P.t1));
        }
        __syncwarp();
    }
}

// d_pos[v].{x, y, w} += the FP64 sums
__global__ void aa_finalize_kernel(int64_t n, const double* __restrict__ acc, float* __restrict__ d_pos) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float* g = d_pos + 4 * i;
        g[0] = __fadd_rn(g[0], (float)acc[3 * i]);
        g[1] = __fadd_rn(g[1], (float)acc[3 * i + 1]);
        g[3] = __fadd_rn(g[3], (float)acc[3 * i + 2]);
    }
}

}  // namespace s2c

using namespace s2c;

extern "C" s2c_status s2c_mark_discontinuity_edges(int H, int W, int B, int V, const float* pos, int T,
                                                   const int32_t* tri, int E, const int32_t* edges,
                                                   const int32_t* edge2tri, int32_t* prim_ids, float* normals,
                                                   s2c_stream stream) {
    S2C_REQUIRE(H > 0 && W > 0 && B > 0 && V >= 0 && T >= 0 && E >= 0, "mark_discontinuity_edges: bad sizes");
    const int64_t BE = (int64_t)B * E;
    S2C_REQUIRE(BE < (1LL << 31), "mark_discontinuity_edges: B*E too large");
    if (BE == 0) return S2C_OK;
    S2C_REQUIRE(pos && edges && edge2tri && prim_ids && normals && (T == 0 || tri),
                "mark_discontinuity_edges: null pointer");
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)edges & 7) == 0 && ((uintptr_t)edge2tri & 7) == 0 &&
                    ((uintptr_t)normals & 7) == 0,
                "mark_discontinuity_edges: misaligned");
    Mesh M;
    M.pos4 = (const float4*)pos;
    M.tri = tri;
    M.edges = (const int2*)edges;
    M.e2t = (const int2*)edge2tri;
    M.V = V;
    M.T = T;
    M.E = E;
    M.divE = FastDiv((uint32_t)E);
    mark_edges_kernel<<<grid_for(BE, 256), 256, 0, (cudaStream_t)stream>>>(H, W, B, M, prim_ids, (float2*)normals);
    S2C_CHECK_LAUNCH("mark_edges_kernel");
    return S2C_OK;
}

static s2c_status aa_backward(int64_t F, const int32_t* frag_pix, const float* frag_attrs, int B, int H, int W,
                              int S, const int32_t* bitset, const int32_t* target, int V, const float* pos, int E,
                              const int32_t* edges, const float* normals, const int32_t* edge2cluster,
                              float* d_pos, float kernel_radius, float rho, void* ws, size_t ws_bytes,
                              cudaStream_t stream) {
    S2C_REQUIRE(F >= 0 && B > 0 && H > 0 && W > 0 && S > 0 && V >= 0 && E >= 0,
                "backward_antialiased_cluster_bitset: bad sizes");
    if (F == 0) return S2C_OK;
    S2C_REQUIRE(frag_pix && frag_attrs && bitset && target && pos && edges && normals && edge2cluster && d_pos,
                "backward_antialiased_cluster_bitset: null pointer");
    S2C_REQUIRE(((uintptr_t)frag_attrs & 15) == 0 && ((uintptr_t)pos & 15) == 0 && ((uintptr_t)normals & 7) == 0 &&
                    ((uintptr_t)edges & 7) == 0,
                "backward_antialiased_cluster_bitset: misaligned");
    S2C_REQUIRE(kernel_radius >= 0.f && kernel_radius < 1024.f, "backward_antialiased_cluster_bitset: bad kernel_radius");
    const int64_t BV = (int64_t)B * V;
    if (ws) {
        S2C_REQUIRE(((uintptr_t)ws & 7) == 0 && ws_bytes >= (size_t)BV * 3 * sizeof(double),
                    "backward_antialiased_cluster_bitset: workspace of %zu bytes, need %lld", ws_bytes,
                    (long long)(BV * 3 * sizeof(double)));
        cudaError_t e = cudaMemsetAsync(ws, 0, (size_t)BV * 3 * sizeof(double), stream);
        if (e != cudaSuccess) return cuda_status(e, "backward_antialiased_cluster_bitset: memset");
    }
    AAArgs A;
    A.F = F;
    A.frag_pix = frag_pix;
    A.frag_attrs = (const float4*)frag_attrs;
    A.B = B;
    A.H = H;
    A.W = W;
    A.S = S;
    A.bitset = bitset;
    A.target = target;
    A.pos4 = (const float4*)pos;
    A.V = V;
    A.E = E;
    A.edges = (const int2*)edges;
    A.normals = (const float2*)normals;
    A.e2c = edge2cluster;
    A.d_pos = d_pos;
    A.acc64 = (double*)ws;
    A.kr = kernel_radius;
    A.rho = rho;
    const int64_t warps = std::min<int64_t>(F, (int64_t)num_sms() * 64);
    aa_backward_kernel<<<grid_for(warps * 32, 256), 256, 0, stream>>>(A);
    S2C_CHECK_LAUNCH("aa_backward_kernel");
    if (ws && BV > 0) {
        aa_finalize_kernel<<<grid_for(BV, 256, (int64_t)num_sms() * 8), 256, 0, stream>>>(BV, (const double*)ws, d_pos);
        S2C_CHECK_LAUNCH("aa_finalize_kernel");
    }
    return S2C_OK;
}

extern "C" s2c_status s2c_backward_antialiased_cluster_bitset(int64_t F, const int32_t* frag_pix,
                                                              const float* frag_attrs, int B, int H, int W, int S,
                                                              const int32_t* bitset, const int32_t* target, int V,
                                                              const float* pos, int E, const int32_t* edges,
                                                              const float* normals, const int32_t* edge2cluster,
                                                              float* d_pos, float kernel_radius, float rho,
                                                              s2c_stream stream) {
    return aa_backward(F, frag_pix, frag_attrs, B, H, W, S, bitset, target, V, pos, E, edges, normals, edge2cluster,
                       d_pos, kernel_radius, rho, nullptr, 0, (cudaStream_t)stream);
}

extern "C" size_t s2c_backward_antialiased_cluster_bitset_workspace_size(int B, int V) {
    return (size_t)(B > 0 ? B : 0) * (size_t)(V > 0 ? V : 0) * 3 * sizeof(double);
}

extern "C" s2c_status s2c_backward_antialiased_cluster_bitset_f64(
    int64_t F, const int32_t* frag_pix, const float* frag_attrs, int B, int H, int W, int S, const int32_t* bitset,
    const int32_t* target, int V, const float* pos, int E, const int32_t* edges, const float* normals,
    const int32_t* edge2cluster, float* d_pos, float kernel_radius, float rho, void* workspace,
    size_t workspace_bytes, s2c_stream stream) {
    S2C_REQUIRE(workspace, "backward_antialiased_cluster_bitset_f64: null workspace");
    return aa_backward(F, frag_pix, frag_attrs, B, H, W, S, bitset, target, V, pos, E, edges, normals, edge2cluster,
                       d_pos, kernel_radius, rho, workspace, workspace_bytes, (cudaStream_t)stream);
}

namespace {
struct AAWs {
    double* acc;
    int32_t* chunks;
    int32_t* prefix;
    int64_t* total;
    void* scan;
    AAEdgeRec* recs;
};

size_t aa_carve(int B, int V, int E, void* base, size_t cap, AAWs* w) {
    Carver cv(base, cap);
    AAWs a;
    const int64_t BE = std::max<int64_t>((int64_t)(B > 0 ? B : 0) * (E > 0 ? E : 0), 1);
    a.acc = cv.take<double>((size_t)(B > 0 ? B : 0) * (size_t)(V > 0 ? V : 0) * 3);
    a.chunks = cv.take<int32_t>(BE);
    a.prefix = cv.take<int32_t>(BE);
    a.total = cv.take<int64_t>(1);
    a.scan = cv.take<char>(scan_workspace_bytes(BE));
    a.recs = cv.take<AAEdgeRec>(BE);
    if (w) *w = a;
    return cv.off;
}
}  // namespace

extern "C" size_t s2c_antialiased_cluster_bitset_grad_planes_workspace_size(int B, int V, int E) {
    return aa_carve(B, V, E, nullptr, (size_t)-1, nullptr) + 256;
}

extern "C" s2c_status s2c_antialiased_cluster_bitset_grad_planes(
    int B, int H, int W, int S, const uint32_t* bitset_planes, const uint32_t* target_planes, int V, const float* pos,
    int T, const int32_t* tri, int E, const int32_t* edges, const int32_t* edge2tri, const int32_t* edge2cluster,
    float* d_pos, float kernel_radius, float rho, void* workspace, size_t workspace_bytes, s2c_stream stream) {
    S2C_REQUIRE(B > 0 && H > 0 && W > 0 && S > 0 && V >= 0 && T >= 0 && E >= 0,
                "antialiased_cluster_bitset_grad: bad sizes");
    const int64_t BE = (int64_t)B * E, BV = (int64_t)B * V;
    S2C_REQUIRE(BE < (1LL << 31), "antialiased_cluster_bitset_grad: B*E too large");
    if (BE == 0 || BV == 0) return S2C_OK;
    S2C_REQUIRE(bitset_planes && target_planes && pos && edges && edge2tri && edge2cluster && d_pos &&
                    (T == 0 || tri) && workspace,
                "antialiased_cluster_bitset_grad: null pointer");
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)edges & 7) == 0 && ((uintptr_t)edge2tri & 7) == 0 &&
                    ((uintptr_t)workspace & 15) == 0,
                "antialiased_cluster_bitset_grad: misaligned");
    S2C_REQUIRE(kernel_radius >= 0.f && kernel_radius < 1024.f, "antialiased_cluster_bitset_grad: bad kernel_radius");
    AAWs ws;
    const size_t need = aa_carve(B, V, E, workspace, workspace_bytes, &ws);
    S2C_REQUIRE(need <= workspace_bytes, "antialiased_cluster_bitset_grad: workspace of %zu bytes, need %zu",
                workspace_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(ws.acc, 0, (size_t)BV * 3 * sizeof(double), st);
    if (e != cudaSuccess) return cuda_status(e, "antialiased_cluster_bitset_grad: memset");
    Mesh M;
    M.pos4 = (const float4*)pos;
    M.tri = tri;
    M.edges = (const int2*)edges;
    M.e2t = (const int2*)edge2tri;
    M.V = V;
    M.T = T;
    M.E = E;
    M.divE = FastDiv((uint32_t)E);
    AAArgs A{};
    A.F = 0;
    A.B = B;
    A.H = H;
    A.W = W;
    A.S = S;
    A.pos4 = (const float4*)pos;
    A.V = V;
    A.E = E;
    A.edges = (const int2*)edges;
    A.e2c = edge2cluster;
    A.d_pos = d_pos;
    A.acc64 = ws.acc;
    A.pplanes = bitset_planes;
    A.tplanes = target_planes;
    A.WQ = (W + 31) / 32;
    A.kr = kernel_radius;
    A.rho = rho;
    aa_count_kernel<<<grid_for(BE, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(A, M, ws.chunks, ws.recs);
    S2C_CHECK_LAUNCH("aa_count_kernel");
    s2c_status ss = inclusive_scan_i32(ws.chunks, BE, ws.prefix, ws.scan, ws.total, st);
    if (ss != S2C_OK) return ss;
    aa_frag_kernel<<<num_sms() * 8, 256, 0, st>>>(A, ws.recs, (const uint32_t*)ws.prefix, ws.total);
    S2C_CHECK_LAUNCH("aa_frag_kernel");
    aa_finalize_kernel<<<grid_for(BV, 256, (int64_t)num_sms() * 8), 256, 0, st>>>(BV, ws.acc, d_pos);
    S2C_CHECK_LAUNCH("aa_finalize_kernel");
    return S2C_OK;
}

extern "C" size_t s2c_antialiased_cluster_bitset_grad_workspace_size(int B, int V, int H, int W, int S, int E) {
    const size_t planes = s2c_bitset_planes_size(B, H, W, S);
    return align_up(s2c_antialiased_cluster_bitset_grad_planes_workspace_size(B, V, E), 256) +
           2 * align_up(planes, 256);
}

extern "C" s2c_status s2c_antialiased_cluster_bitset_grad(int B, int H, int W, int S, const int32_t* bitset,
                                                          const int32_t* target, int V, const float* pos, int T,
                                                          const int32_t* tri, int E, const int32_t* edges,
                                                          const int32_t* edge2tri, const int32_t* edge2cluster,
                                                          float* d_pos, float kernel_radius, float rho,
                                                          void* workspace, size_t workspace_bytes,
                                                          s2c_stream stream) {
    S2C_REQUIRE(B > 0 && H > 0 && W > 0 && S > 0, "antialiased_cluster_bitset_grad: bad sizes");
    S2C_REQUIRE(bitset && target && workspace, "antialiased_cluster_bitset_grad: null pointer");
    const size_t need = s2c_antialiased_cluster_bitset_grad_workspace_size(B, V, H, W, S, E);
    S2C_REQUIRE(workspace_bytes >= need, "antialiased_cluster_bitset_grad: workspace of %zu bytes, need %zu",
                workspace_bytes, need);
    const size_t acc = align_up(s2c_antialiased_cluster_bitset_grad_planes_workspace_size(B, V, E), 256);
    const size_t planes = align_up(s2c_bitset_planes_size(B, H, W, S), 256);
    uint32_t* pp = (uint32_t*)((char*)workspace + acc);
    uint32_t* tp = (uint32_t*)((char*)workspace + acc + planes);
    s2c_status s = s2c_bitset_to_planes(B, H, W, S, bitset, pp, stream);
    if (s == S2C_OK) s = s2c_bitset_to_planes(B, H, W, S, target, tp, stream);
    if (s != S2C_OK) return s;
    return s2c_antialiased_cluster_bitset_grad_planes(B, H, W, S, pp, tp, V, pos, T, tri, E, edges, edge2tri,
                                                      edge2cluster, d_pos, kernel_radius, rho, workspace, acc,
                                                      stream);
}
