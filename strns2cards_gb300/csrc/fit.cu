// Batched per-cluster card fitting in one persistent launch (s2c_fit_iteration).
//
// The reference fits the cards of a hair model cluster by cluster (3_fitting.py:381-406):
// per cluster, the strands' target coverage (dda_compute_fragments +
// cluster_mask_from_fragments), the card raster (compute_fragments + the mask), the
// antialiased-bitset gradient (antialias.cu:121-317) and a Laplacian-regularised step.
// Here one launch advances every cluster by one iteration.  Each cluster is framed at H x W
// with one bit plane per image (bit x % 32 of word y * WQ + x / 32 = pixel (y, x)), small
// enough for shared memory (512 x 128 px: 8 KB), so nothing of an image leaves the SM:
//
//  * CTAs take (cluster, segment chunk) items from a queue, largest clusters first, and
//    rasterise the chunk's strand segments with the reference's exact DDA arithmetic into a
//    shared target plane; a cluster split into several chunks ORs its partial planes into
//    an L2-resident plane, and the CTA that completes the cluster's last chunk (a counter,
//    no waiting) carries on with it;
//  * that CTA then rasterises the cluster's card (the reference's FP32 coverage test, all
//    triangles OR-ed) into a second shared plane, marks the silhouette / boundary edges,
//    regenerates their DDA fragments, evaluates each fragment's Gaussian window over the
//    two planes where they differ and accumulates the chain-rule contributions per card
//    vertex in FP64 shared-memory atomics, takes the normalised gradient step and the
//    Jacobi Laplacian steps in shared memory, and writes the card back.
//
// The same iteration as the per-cluster call sequence (fused DDA -> bitset, fused card
// raster, antialias backward, step, card_laplacian_smooth): coverage bit for bit, the
// gradient's FP64 sums in another order.
#include <algorithm>

#include "aa.cuh"
#include "common.cuh"
#include "tri.cuh"

namespace s2c {

struct FitArgs {
    int C, H, W, WQ;
    // strands: positions (C, Vs) -- or, with voff, cluster c's vertices at
    // [voff[c], voff[c + 1]) of one packed array -- and one shared polyline edge list;
    // edge_ids[i] = c * Es + e grouped by cluster, cluster c owning [coff[c], coff[c + 1])
    const float4* __restrict__ spos;
    const int32_t* __restrict__ voff;
    int Vs, Es;
    const int2* __restrict__ sedges;
    const int32_t* __restrict__ edge_ids;
    const int32_t* __restrict__ coff;
    // cards: positions (C, Vc) updated in place, one shared topology
    float4* __restrict__ cpos;
    int Vc, Tc, Ec, nadj;
    const int* __restrict__ ctri;
    const int2* __restrict__ cedges;
    const int2* __restrict__ ce2t;
    const int32_t* __restrict__ lap_off;   // (Vc + 1) CSR of one card's neighbours
    const int32_t* __restrict__ lap_adj;
    // work: (cluster, chunk) items in processing order, chunks per cluster
    const int2* __restrict__ items;
    int n_items, chunk;
    const int32_t* __restrict__ nchunks;
    uint32_t* __restrict__ gplanes;        // (C, H, WQ) partial target planes, zero at launch
    int* __restrict__ ctrl;                // [0] queue head, [1 + c] chunks of cluster c done
    // the step: x, y -= g * (step_scale / max |g|); then nlap Jacobi steps with weight lam
    float step_scale, lam, kr, rho;
    int nlap, aa_warp;                      // aa_warp: one warp per fragment (else one thread)
};

struct SmemPos {
    const float4* p;
    __device__ __forceinline__ float4 operator()(int v) const { return p[v]; }
};

struct FitSmem {
    uint32_t* tplane;
    uint32_t* pplane;
    double* acc;     // (Vc, 3): d/dx, d/dy, d/dw
    float4* P;       // card positions
    float* L0;       // (Vc, 3) Laplacian ping-pong
    float* L1;
    int32_t* epre;   // (Ec) inclusive prefix of silhouette fragment counts
    float2* enrm;
    int32_t* loff;
    int32_t* ladj;
};

__host__ __device__ inline size_t fit_smem_bytes(int H, int WQ, int Vc, int Ec, int nadj, FitSmem* s, char* base) {
    size_t off = 0;
    auto take = [&](size_t bytes, size_t align) {
        off = (off + align - 1) / align * align;
        char* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    };
    char* t = take((size_t)H * WQ * 4, 16);
    char* pp = take((size_t)H * WQ * 4, 16);
    char* acc = take((size_t)Vc * 3 * 8, 16);
    char* P = take((size_t)Vc * 16, 16);
    char* L0 = take((size_t)Vc * 12, 16);
    char* L1 = take((size_t)Vc * 12, 16);
    char* ep = take((size_t)Ec * 4, 16);
    char* en = take((size_t)Ec * 8, 16);
    char* lo = take((size_t)(Vc + 1) * 4, 16);
    char* la = take((size_t)(nadj > 1 ? nadj : 1) * 4, 16);
    if (s) {
        s->tplane = (uint32_t*)t;
        s->pplane = (uint32_t*)pp;
        s->acc = (double*)acc;
        s->P = (float4*)P;
        s->L0 = (float*)L0;
        s->L1 = (float*)L1;
        s->epre = (int32_t*)ep;
        s->enrm = (float2*)en;
        s->loff = (int32_t*)lo;
        s->ladj = (int32_t*)la;
    }
    return (off + 15) / 16 * 16;
}

__device__ __forceinline__ void plane_set(uint32_t* plane, int WQ, int y, int x) {
    atomicOr(plane + y * WQ + (x >> 5), 1u << (x & 31));
}

__device__ __forceinline__ int plane_get(const uint32_t* plane, int WQ, int y, int x) {
    return (plane[y * WQ + (x >> 5)] >> (x & 31)) & 1;
}

// The DDA fragments of strand segment eid (dda.cu:9-225: bounds and depth tests included)
// into the target plane of cluster c; ids of another cluster or out of range are skipped.
__device__ __forceinline__ void fit_cover_segment(const FitArgs& a, int c, int32_t eid, uint32_t* plane) {
    if (eid < 0 || eid >= a.C * a.Es) return;
    const int b = eid / a.Es;
    if (b != c) return;
    const int e = eid - b * a.Es;
    const int pr = prim_roundtrip(e);       // the reference carries the id as float(e + 1)
    if (pr < 0 || pr >= a.Es) return;
    const int2 ev = __ldg(a.sedges + e);
    int64_t v0 = (int64_t)b * a.Vs;
    int nv = a.Vs;
    if (a.voff) {
        v0 = __ldg(a.voff + b);
        nv = __ldg(a.voff + b + 1) - (int)v0;
    }
    if ((unsigned)ev.x >= (unsigned)nv || (unsigned)ev.y >= (unsigned)nv) return;
    const float4 p0 = __ldg(a.spos + v0 + ev.x), p1 = __ldg(a.spos + v0 + ev.y);
    const Span s = dda_span(p0, p1, a.H, a.W);
    const bool zfast = depth_always_passes(p0, p1);
    for (int k = 0; k < s.count; ++k) {
        float x, y;
        dda_sample(s, k, x, y);
        const int h = f2i(floorf(y)), w = f2i(floorf(x));
        if (h < 0 || h >= a.H || w < 0 || w >= a.W) continue;
        if (!zfast) {
            const float t1 = dda_t1(p0, p1, x, y, s.axis, a.H, a.W);
            if (!z_ok(dda_z(p0, p1, t1))) continue;
        }
        plane_set(plane, a.WQ, h, w);
    }
}

// Set-up of one silhouette fragment (antialias.cu:121-176, as aa_prep) on the shared planes
struct FitFrag {
    float fx, fy, px, py, pw, t0, t1;
    float2 nrm;
    int2 ev;
    int c01, h0, h1, w0, w1;
};

__device__ __forceinline__ bool fit_frag_prep(const FitArgs& a, const FitSmem& S, int h, int w, float axis, float t1,
                                              int e, float2 nrm, FitFrag& P) {
    const float fH = (float)a.H, fW = (float)a.W;
    if (e < 0 || e >= a.Ec || h < 0 || h >= a.H || w < 0 || w >= a.W) return false;
    const float t0 = __fsub_rn(1.f, t1);
    const int2 ev = __ldg(a.cedges + e);
    if ((unsigned)ev.x >= (unsigned)a.Vc || (unsigned)ev.y >= (unsigned)a.Vc) return false;
    const float4 p0 = S.P[ev.x], p1 = S.P[ev.y];
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
    if (nw < 0 || nw >= a.W || nh < 0 || nh >= a.H || dot == 0.f) return false;
    // one cluster per view: the card's plane is cluster 0's
    const int c01 = 1 - (dot > 0.f ? plane_get(S.pplane, a.WQ, nh, nw) : plane_get(S.pplane, a.WQ, h, w));
    if (c01 == 0) return false;
    const int R = f2i(floorf(a.kr));
    const int cw = f2i(floorf(fx)), ch = f2i(floorf(fy));
    P.h0 = max(ch - R, 0);
    P.h1 = min(ch + R, a.H - 1) + 1;
    P.w0 = max(cw - R, 0);
    P.w1 = min(cw + R, a.W - 1) + 1;
    aa_trim_window(a.kr, fx, fy, P.h0, P.h1, P.w0, P.w1);
    P.fx = fx;
    P.fy = fy;
    P.px = px;
    P.py = py;
    P.pw = pw;
    P.t0 = t0;
    P.t1 = t1;
    P.nrm = nrm;
    P.ev = ev;
    P.c01 = c01;
    return true;
}

// One window row of a fragment (antialias.cu:177-279): the 1-2 plane words covering
// [w0, w1) of both images, visiting only the pixels where they differ, in x order
__device__ __forceinline__ void fit_window_row(const FitArgs& a, const FitSmem& S, const FitFrag& P, const AAWin& q,
                                               int th, float& sum, float& comp) {
    const uint32_t* prow = S.pplane + th * a.WQ;
    const uint32_t* trow = S.tplane + th * a.WQ;
    const float dy = __fsub_rn(__fadd_rn((float)th, 0.5f), P.fy);
    const int q0 = P.w0 >> 5, width = P.w1 - P.w0;
    if (width <= 32) {
        // the row as one 32-bit mask from w0 (one flat pixel loop, as aa_window_row)
        const int sh = P.w0 & 31;
        uint64_t pv = prow[q0], tv = trow[q0];
        if (sh + width > 32) {
            pv |= (uint64_t)prow[q0 + 1] << 32;
            tv |= (uint64_t)trow[q0 + 1] << 32;
        }
        const uint32_t m = width == 32 ? 0xffffffffu : (1u << width) - 1u;
        const uint32_t pw = (uint32_t)(pv >> sh) & m, tw = (uint32_t)(tv >> sh) & m;
        const uint32_t pos = pw & ~tw;
        uint32_t any = pw ^ tw;
        while (any) {
            const int bit = __ffs(any) - 1;
            any &= any - 1;
            const float dx = __fsub_rn(__fadd_rn((float)(P.w0 + bit), 0.5f), P.fx);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < q.kr2)) continue;
            const float wgt = __fmul_rn(q.cc, expf(-q.alpha * n2));
            kahan_add(sum, comp, ((pos >> bit) & 1u) ? __fmul_rn(wgt, a.rho) : -wgt);
        }
        return;
    }
    for (int qq = q0; qq <= (P.w1 - 1) >> 5; ++qq) {
        const int lo = max(P.w0 - 32 * qq, 0), hi = min(P.w1 - 32 * qq, 32);
        const uint32_t m = (hi == 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
        const uint32_t pv = prow[qq], tv = trow[qq];
        const uint32_t pos = pv & ~tv & m;
        uint32_t any = (pv ^ tv) & m;
        while (any) {
            const int bit = __ffs(any) - 1;
            any &= any - 1;
            const float dx = __fsub_rn(__fadd_rn((float)(32 * qq + bit), 0.5f), P.fx);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < q.kr2)) continue;
            const float wgt = __fmul_rn(q.cc, expf(-q.alpha * n2));
            kahan_add(sum, comp, ((pos >> bit) & 1u) ? __fmul_rn(wgt, a.rho) : -wgt);
        }
    }
}

// fragment j of the cluster's silhouette edges: its edge (binary search of the prefix), the
// DDA sample and the depth test (dda.cu:146-225), then the set-up; false: no contribution
__device__ __forceinline__ bool fit_locate_frag(const FitArgs& a, const FitSmem& S, int j, FitFrag& P) {
    int lo = 0, hi = a.Ec;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (S.epre[mid] <= j) lo = mid + 1;
        else hi = mid;
    }
    const int e = lo;
    if (e >= a.Ec) return false;
    const int k = j - (e > 0 ? S.epre[e - 1] : 0);
    // an edge with fragments is a marked one, whose vertices are in range
    const int2 ev = __ldg(a.cedges + e);
    const float4 p0 = S.P[ev.x], p1 = S.P[ev.y];
    const Span sp = dda_span(p0, p1, a.H, a.W);
    if (k >= sp.count) return false;
    float x, y;
    dda_sample(sp, k, x, y);
    const int h = f2i(floorf(y)), w = f2i(floorf(x));
    if (h < 0 || h >= a.H || w < 0 || w >= a.W) return false;
    const float t1 = dda_t1(p0, p1, x, y, sp.axis, a.H, a.W);
    if (!z_ok(dda_z(p0, p1, t1))) return false;
    return fit_frag_prep(a, S, h, w, sp.axis, t1, prim_roundtrip(e), S.enrm[e], P);
}

__device__ __forceinline__ void fit_accumulate(const FitArgs& a, const FitSmem& S, const FitFrag& P, float dc) {
    float dpx, dpy, dpw;
    if (!aa_chain_rule(a.H, a.W, dc, P.nrm, P.px, P.py, P.pw, dpx, dpy, dpw)) return;
    double* a0 = S.acc + 3 * P.ev.x;
    double* a1 = S.acc + 3 * P.ev.y;
    atomicAdd(a0 + 0, (double)__fmul_rn(dpx, P.t0));
    atomicAdd(a0 + 1, (double)__fmul_rn(dpy, P.t0));
    atomicAdd(a0 + 2, (double)__fmul_rn(dpw, P.t0));
    atomicAdd(a1 + 0, (double)__fmul_rn(dpx, P.t1));
    atomicAdd(a1 + 1, (double)__fmul_rn(dpy, P.t1));
    atomicAdd(a1 + 2, (double)__fmul_rn(dpw, P.t1));
}

// block-wide inclusive scan of v[0, n) in place
__device__ __forceinline__ void fit_block_scan(int32_t* v, int n, int* s_warp) {
    const int nt = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (n + nt - 1) / nt;
    const int b0 = min(tid * per, n), b1 = min(b0 + per, n);
    int sum = 0;
    for (int i = b0; i < b1; ++i) sum += v[i];
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = nt >> 5;
        const int x = lane < nw ? s_warp[lane] : 0;
        int xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += t;
        }
        if (lane < nw) s_warp[lane] = xi - x;
    }
    __syncthreads();
    int run = s_warp[warp] + inc - sum;
    for (int i = b0; i < b1; ++i) {
        run += v[i];
        v[i] = run;
    }
    __syncthreads();
}

__device__ __forceinline__ float fit_block_max(float m, float* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) s_red[warp] = m;
    __syncthreads();
    float r = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r = fmaxf(r, s_red[i]);
    __syncthreads();
    return r;
}

// the rest of cluster c's iteration, its target plane in S.tplane
__device__ void fit_tail(const FitArgs& a, const FitSmem& S, int c, int* s_misc, float* s_red) {
    const int nt = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int PW = a.H * a.WQ;
    float4* cp = a.cpos + (int64_t)c * a.Vc;
    for (int v = tid; v < a.Vc; v += nt) {
        S.P[v] = cp[v];
        S.acc[3 * v] = S.acc[3 * v + 1] = S.acc[3 * v + 2] = 0.0;
    }
    for (int j = tid; j < PW; j += nt) S.pplane[j] = 0u;
    if (tid == 0) s_misc[0] = 0;
    __syncthreads();
    // card raster: warps take triangles, lanes the pixels of the bounding rectangle
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(s_misc, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.Tc) break;
        float4 P3[3];
        bool ok[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int v = __ldg(a.ctri + 3 * t + i);
            ok[i] = (unsigned)v < (unsigned)a.Vc;
            P3[i] = ok[i] ? S.P[v] : make_float4(0.f, 0.f, 0.f, 1.f);
        }
        const int4 rc = tri_rect_of(a.H, a.W, P3, ok);
        const int area = rc.y * rc.w;
        if (area <= 0) continue;
        int yy = lane / rc.w, xx = lane - yy * rc.w;
        const int dy = 32 / rc.w, dx = 32 - dy * rc.w;
        for (int q = lane; q < area; q += 32) {
            const int y = rc.x + yy, x = rc.z + xx;
            yy += dy;
            xx += dx;
            if (xx >= rc.w) {
                xx -= rc.w;
                ++yy;
            }
            const TriEdges e = tri_edges(P3[0], P3[1], P3[2], ndc_of(x, (float)a.W), ndc_of(y, (float)a.H));
            if (tri_surely_outside(e)) continue;
            float b0, b1, z;
            if (tri_finish(e, P3[0], P3[1], P3[2], b0, b1, z)) plane_set(S.pplane, a.WQ, y, x);
        }
    }
    __syncthreads();
    // silhouette / boundary edges (antialias.cu:38-94) and their DDA fragment counts
    for (int e = tid; e < a.Ec; e += nt) {
        float2 nrm = make_float2(0.f, 0.f);
        const int2 ev = __ldg(a.cedges + e);
        const int m = mark_edge_t(a.H, a.W, ev, __ldg(a.ce2t + e), a.ctri, a.Tc, a.Vc, SmemPos{S.P}, nrm);
        S.enrm[e] = nrm;
        S.epre[e] = m == 2 ? dda_span(S.P[ev.x], S.P[ev.y], a.H, a.W).count : 0;
    }
    __syncthreads();
    fit_block_scan(S.epre, a.Ec, s_misc + 1);
    const int F = a.Ec > 0 ? S.epre[a.Ec - 1] : 0;
    const AAWin win = aa_win(a.kr);
    if (a.aa_warp) {
        // one warp per fragment: lanes take the window rows
        for (int j = warp; j < F; j += nt >> 5) {
            FitFrag P;
            if (!fit_locate_frag(a, S, j, P)) continue;
            float sum = 0.f, comp = 0.f;
            if (P.w1 > P.w0)
                for (int th = P.h0 + lane; th < P.h1; th += 32) fit_window_row(a, S, P, win, th, sum, comp);
            const float dc = __fmul_rn((float)P.c01, warp_sum_comp(sum, comp));
            if (lane == 0 && dc != 0.f) fit_accumulate(a, S, P, dc);
        }
    } else {
        for (int j = tid; j < F; j += nt) {
            FitFrag P;
            if (!fit_locate_frag(a, S, j, P)) continue;
            float sum = 0.f, comp = 0.f;
            if (P.w1 > P.w0)
                for (int th = P.h0; th < P.h1; ++th) fit_window_row(a, S, P, win, th, sum, comp);
            const float dc = __fmul_rn((float)P.c01, __fsub_rn(sum, comp));
            if (dc != 0.f) fit_accumulate(a, S, P, dc);
        }
    }
    __syncthreads();
    // normalised step on x, y: the largest |d_pos| moves step_scale (x, y -= g / max|g| * s)
    float m = 0.f;
    for (int v = tid; v < a.Vc; v += nt)
        m = fmaxf(m, fmaxf(fabsf(__double2float_rn(S.acc[3 * v])), fabsf(__double2float_rn(S.acc[3 * v + 1]))));
    m = fit_block_max(m, s_red);
    const float scale = __fmul_rn(__fdiv_rn(1.f, fmaxf(m, 1e-30f)), a.step_scale);
    for (int v = tid; v < a.Vc; v += nt) {
        const float4 p = S.P[v];
        S.L0[3 * v] = __fsub_rn(p.x, __fmul_rn(__double2float_rn(S.acc[3 * v]), scale));
        S.L0[3 * v + 1] = __fsub_rn(p.y, __fmul_rn(__double2float_rn(S.acc[3 * v + 1]), scale));
        S.L0[3 * v + 2] = p.z;
    }
    __syncthreads();
    // Jacobi Laplacian steps (as card_laplacian_kernel): p <- p - lam (p - mean(neighbours))
    float* src = S.L0;
    float* dst = S.L1;
    for (int st = 0; st < a.nlap; ++st) {
        for (int v = tid; v < a.Vc; v += nt) {
            float x = src[3 * v], y = src[3 * v + 1], z = src[3 * v + 2];
            const int o0 = S.loff[v], o1 = S.loff[v + 1];
            if (o1 > o0) {
                float sx = 0.f, sy = 0.f, sz = 0.f;
                for (int q = o0; q < o1; ++q) {
                    const int u = S.ladj[q];
                    if ((unsigned)u >= (unsigned)a.Vc) continue;
                    sx = __fadd_rn(sx, src[3 * u]);
                    sy = __fadd_rn(sy, src[3 * u + 1]);
                    sz = __fadd_rn(sz, src[3 * u + 2]);
                }
                const float dg = (float)(o1 - o0);
                x = __fsub_rn(x, __fmul_rn(a.lam, __fsub_rn(x, __fdiv_rn(sx, dg))));
                y = __fsub_rn(y, __fmul_rn(a.lam, __fsub_rn(y, __fdiv_rn(sy, dg))));
                z = __fsub_rn(z, __fmul_rn(a.lam, __fsub_rn(z, __fdiv_rn(sz, dg))));
            }
            dst[3 * v] = x;
            dst[3 * v + 1] = y;
            dst[3 * v + 2] = z;
        }
        __syncthreads();
        float* t = src;
        src = dst;
        dst = t;
    }
    for (int v = tid; v < a.Vc; v += nt) cp[v] = make_float4(src[3 * v], src[3 * v + 1], src[3 * v + 2], S.P[v].w);
}

__global__ void __launch_bounds__(1024) fit_kernel(FitArgs a) {
    extern __shared__ __align__(16) unsigned char fit_smem[];
    __shared__ int s_item, s_last;
    __shared__ int s_misc[40];
    __shared__ float s_red[32];
    FitSmem S;
    fit_smem_bytes(a.H, a.WQ, a.Vc, a.Ec, a.nadj, &S, (char*)fit_smem);
    const int nt = blockDim.x, tid = threadIdx.x;
    const int PW = a.H * a.WQ;
    for (int v = tid; v <= a.Vc; v += nt) S.loff[v] = __ldg(a.lap_off + v);
    for (int q = tid; q < a.nadj; q += nt) S.ladj[q] = __ldg(a.lap_adj + q);
    for (;;) {
        if (tid == 0) s_item = atomicAdd(a.ctrl, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= a.n_items) break;
        const int2 it = __ldg(a.items + item);
        const int c = it.x, k = it.y;
        for (int j = tid; j < PW; j += nt) S.tplane[j] = 0u;
        __syncthreads();
        const int s0 = __ldg(a.coff + c) + k * a.chunk;
        const int s1 = min(__ldg(a.coff + c + 1), s0 + a.chunk);
        for (int i = s0 + tid; i < s1; i += nt) fit_cover_segment(a, c, __ldg(a.edge_ids + i), S.tplane);
        __syncthreads();
        if (__ldg(a.nchunks + c) > 1) {
            uint32_t* g = a.gplanes + (int64_t)c * PW;
            for (int j = tid; j < PW; j += nt) {
                const uint32_t v = S.tplane[j];
                if (v) atomicOr(g + j, v);
            }
            __threadfence();
            __syncthreads();
            if (tid == 0) s_last = atomicAdd(a.ctrl + 1 + c, 1) == __ldg(a.nchunks + c) - 1;
            __syncthreads();
            if (!s_last) continue;
            __threadfence();
            for (int j = tid; j < PW; j += nt) S.tplane[j] = __ldcg(g + j);
            __syncthreads();
        }
        fit_tail(a, S, c, s_misc, s_red);
        __syncthreads();
    }
}

}  // namespace s2c

using namespace s2c;

namespace {
constexpr int kFitMaxWords = 16384;   // H * ceil(W / 32) per plane (64 KB)
constexpr int kFitMaxVerts = 2048;
constexpr int kFitMaxEdges = 8192;
}  // namespace

extern "C" size_t s2c_fit_smem_bytes(int H, int W, int Vc, int Ec, int nadj) {
    if (H <= 0 || W <= 0 || Vc < 0 || Ec < 0 || nadj < 0) return 0;
    return fit_smem_bytes(H, (W + 31) / 32, Vc, Ec, nadj, nullptr, nullptr);
}

extern "C" size_t s2c_fit_workspace_size(int C, int H, int W) {
    if (C <= 0 || H <= 0 || W <= 0) return 0;
    Carver cv(nullptr, (size_t)-1);
    cv.take<int>((size_t)C + 1);
    cv.take<uint32_t>((size_t)C * H * ((W + 31) / 32));
    return cv.off + 256;
}

extern "C" s2c_status s2c_fit_iteration(int C, int H, int W, int Vs, const float* strand_pos,
                                        const int32_t* vert_offsets, int Es,
                                        const int32_t* strand_edges, const int32_t* edge_ids,
                                        const int32_t* cluster_offsets, int Vc, float* card_pos, int Tc,
                                        const int32_t* card_tri, int Ec, const int32_t* card_edges,
                                        const int32_t* card_edge2tri, const int32_t* lap_offsets,
                                        const int32_t* lap_adj, int nadj, const int32_t* items, int n_items,
                                        int chunk, const int32_t* chunks_per_cluster, float step_scale, float lam,
                                        int laplacian_steps, float kernel_radius, float rho, int threads,
                                        int ctas_per_sm, int aa_warp, void* workspace, size_t workspace_bytes,
                                        s2c_stream stream) {
    S2C_REQUIRE(C > 0 && H > 0 && W > 0 && Vs >= 0 && Es >= 0 && Vc > 0 && Tc >= 0 && Ec >= 0 && nadj >= 0,
                "fit_iteration: bad sizes");
    const int WQ = (W + 31) / 32;
    S2C_REQUIRE((int64_t)H * WQ <= kFitMaxWords, "fit_iteration: a %dx%d frame exceeds %d plane words", H, W,
                kFitMaxWords);
    S2C_REQUIRE(Vc <= kFitMaxVerts && Ec <= kFitMaxEdges, "fit_iteration: cards of at most %d vertices and %d edges",
                kFitMaxVerts, kFitMaxEdges);
    S2C_REQUIRE((int64_t)C * Es < (1LL << 31), "fit_iteration: C * Es too large");
    S2C_REQUIRE(threads == 128 || threads == 256 || threads == 512 || threads == 1024,
                "fit_iteration: threads must be 128, 256, 512 or 1024");
    S2C_REQUIRE(ctas_per_sm >= 1 && ctas_per_sm <= 16 && chunk > 0 && n_items >= 0 && laplacian_steps >= 0,
                "fit_iteration: bad launch parameters");
    S2C_REQUIRE(kernel_radius >= 0.f && kernel_radius < 1024.f, "fit_iteration: bad kernel_radius");
    S2C_REQUIRE(strand_pos && strand_edges && cluster_offsets && card_pos && card_edges && card_edge2tri &&
                    lap_offsets && (Tc == 0 || card_tri) && (nadj == 0 || lap_adj) && (n_items == 0 || items) &&
                    chunks_per_cluster && workspace,
                "fit_iteration: null pointer");
    S2C_REQUIRE(((uintptr_t)strand_pos & 15) == 0 && ((uintptr_t)card_pos & 15) == 0 &&
                    ((uintptr_t)strand_edges & 7) == 0 && ((uintptr_t)card_edges & 7) == 0 &&
                    ((uintptr_t)card_edge2tri & 7) == 0 && ((uintptr_t)items & 7) == 0,
                "fit_iteration: misaligned");
    const size_t need = s2c_fit_workspace_size(C, H, W);
    if (workspace_bytes < need) {
        set_error("fit_iteration: workspace of %zu bytes, need %zu", workspace_bytes, need);
        return S2C_ERR_WORKSPACE;
    }
    Carver cv(workspace, workspace_bytes);
    int* ctrl = cv.take<int>((size_t)C + 1);
    uint32_t* gplanes = cv.take<uint32_t>((size_t)C * H * WQ);
    cudaStream_t st = (cudaStream_t)stream;
    // the queue head, the per-cluster chunk counters and the partial planes start at zero
    cudaError_t e = cudaMemsetAsync(workspace, 0, cv.off, st);
    if (e != cudaSuccess) return cuda_status(e, "fit_iteration: clearing the workspace");
    if (n_items == 0) return S2C_OK;
    const size_t smem = fit_smem_bytes(H, WQ, Vc, Ec, nadj, nullptr, nullptr);
    S2C_REQUIRE(smem <= 200 * 1024, "fit_iteration: %zu bytes of shared memory per CTA (frame, card and edges)", smem);
    static std::atomic<size_t> cfg[kMaxDevices];
    const int slot = current_device_slot();
    if (smem > cfg[slot].load()) {
        cudaFuncSetAttribute(fit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cfg[slot].store(smem);
    }
    FitArgs a;
    a.C = C;
    a.H = H;
    a.W = W;
    a.WQ = WQ;
    a.spos = (const float4*)strand_pos;
    a.voff = vert_offsets;
    a.Vs = Vs;
    a.Es = Es;
    a.sedges = (const int2*)strand_edges;
    a.edge_ids = edge_ids;
    a.coff = cluster_offsets;
    a.cpos = (float4*)card_pos;
    a.Vc = Vc;
    a.Tc = Tc;
    a.Ec = Ec;
    a.nadj = nadj;
    a.ctri = card_tri;
    a.cedges = (const int2*)card_edges;
    a.ce2t = (const int2*)card_edge2tri;
    a.lap_off = lap_offsets;
    a.lap_adj = lap_adj;
    a.items = (const int2*)items;
    a.n_items = n_items;
    a.chunk = chunk;
    a.nchunks = chunks_per_cluster;
    a.gplanes = gplanes;
    a.ctrl = ctrl;
    a.step_scale = step_scale;
    a.lam = lam;
    a.kr = kernel_radius;
    a.rho = rho;
    a.nlap = laplacian_steps;
    a.aa_warp = aa_warp ? 1 : 0;
    const unsigned grid = (unsigned)std::min<int64_t>((int64_t)ctas_per_sm * num_sms(), n_items);
    fit_kernel<<<grid, threads, smem, st>>>(a);
    S2C_CHECK_LAUNCH("fit_kernel");
    return S2C_OK;
}
