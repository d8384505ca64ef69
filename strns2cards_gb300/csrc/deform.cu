// Card deformation operators.
//
// Laplacian smoothing of card vertices.  The reference builds the uniform Laplacian
// L = D - A of the card edges (optimizer.py:70-99) and uses it as the preconditioner I + lambda L
// (3_fitting.py:347-355) and as the regulariser |L p|^2 (3_fitting.py:359,401); it has no
// smoothing kernel.  The operator here is the explicit Jacobi form on every card's
// quad edges (h_edges + w_edges, 3_fitting.py:319): p <- p - lambda D^-1 L p, i.e.
// p <- p - lambda (p - mean of the neighbours), for a given number of steps.  All cards
// share one grid topology (texture_utils.py:525-599), passed once as a CSR adjacency; a
// CTA stages whole cards in shared memory and runs every step there, so HBM sees one
// read and one write of the vertices.
//
// Linear blend skinning of strand vertices to the 4 nearest guide points (card
// centre-line vertices): y = sum_k w_k (A_k x + t_k), w = softmax(-d_k^2 / tau) over the
// 4 nearest guides at bind time, M_k = [A_k | t_k] row-major 3x4.  Binding: a uniform grid
// over the guides, a shell search per vertex in exact FP32 with ties broken by guide
// index (the same selection as a brute-force scan), then per-guide inverse lists sorted
// by vertex, so the parameter gradient is a per-guide reduction with a fixed order.
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace s2c {
namespace {

// ===================================== Laplacian =======================================
constexpr int kLapThreads = 256;
constexpr int kLapSmem = 48 * 1024;

struct LapArgs {
    int num_cards, nv, cpc, ngroups, nadj, steps;
    const int32_t* off;
    const int32_t* adj;
    const float* in;
    float* out;
    float lam;
};

__global__ void __launch_bounds__(kLapThreads) card_laplacian_kernel(LapArgs a) {
    extern __shared__ __align__(16) int32_t lsm[];
    const int nv = a.nv;
    int32_t* soff = lsm;
    int32_t* sadj = soff + nv + 1;
    float* P0 = (float*)(sadj + a.nadj);
    float* P1 = P0 + 3 * a.cpc * nv;
    const int tid = threadIdx.x;
    for (int k = tid; k <= nv; k += kLapThreads) soff[k] = __ldg(a.off + k);
    for (int k = tid; k < a.nadj; k += kLapThreads) sadj[k] = __ldg(a.adj + k);
    for (int g = blockIdx.x; g < a.ngroups; g += gridDim.x) {
        const int64_t c0 = (int64_t)g * a.cpc;
        const int nc = (int)(a.num_cards - c0 < a.cpc ? a.num_cards - c0 : a.cpc);
        const int n = nc * nv;
        const float* src_g = a.in + 3 * c0 * nv;
        for (int k = tid; k < 3 * n; k += kLapThreads) P0[k] = __ldg(src_g + k);
        __syncthreads();
        float* src = P0;
        float* dst = P1;
        for (int s = 0; s < a.steps; ++s) {
            for (int p = tid; p < n; p += kLapThreads) {
                const int card = p / nv;
                const int v = p - card * nv;
                const int base = card * nv;
                float x = src[3 * p], y = src[3 * p + 1], z = src[3 * p + 2];
                const int o0 = soff[v], o1 = soff[v + 1];
                if (o1 > o0) {
                    float sx = 0.f, sy = 0.f, sz = 0.f;
                    for (int q = o0; q < o1; ++q) {
                        const int lu = sadj[q];
                        if ((unsigned)lu >= (unsigned)nv) continue;
                        const int u = base + lu;
                        sx = __fadd_rn(sx, src[3 * u]);
                        sy = __fadd_rn(sy, src[3 * u + 1]);
                        sz = __fadd_rn(sz, src[3 * u + 2]);
                    }
                    const float dg = (float)(o1 - o0);
                    x = __fsub_rn(x, __fmul_rn(a.lam, __fsub_rn(x, __fdiv_rn(sx, dg))));
                    y = __fsub_rn(y, __fmul_rn(a.lam, __fsub_rn(y, __fdiv_rn(sy, dg))));
                    z = __fsub_rn(z, __fmul_rn(a.lam, __fsub_rn(z, __fdiv_rn(sz, dg))));
                }
                dst[3 * p] = x;
                dst[3 * p + 1] = y;
                dst[3 * p + 2] = z;
            }
            __syncthreads();
            float* t = src;
            src = dst;
            dst = t;
        }
        float* out_g = a.out + 3 * c0 * nv;
        for (int k = tid; k < 3 * n; k += kLapThreads) out_g[k] = src[k];
        __syncthreads();
    }
}

// ======================================== LBS ==========================================
constexpr int kMaxCells = 1 << 22;

struct GridDesc {
    float lo[3];
    float cell, inv_cell;
    int n[3];
};

__device__ __forceinline__ float d2_of(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// cell index along one axis, unclamped (saturated at +-1e6; NaN -> 0)
__device__ __forceinline__ int cell_coord(float v, float lo, float inv) {
    const float c = floorf(__fmul_rn(__fsub_rn(v, lo), inv));
    return c < -1e6f ? -1000000 : (c > 1e6f ? 1000000 : f2i(c));
}

// one CTA: guide bounding box and grid shape (about two guides per cell)
__global__ void __launch_bounds__(1024) lbs_grid_kernel(int G, const float* __restrict__ g, int max_cells,
                                                         GridDesc* __restrict__ gd) {
    __shared__ float red[6][32];
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < G; i += blockDim.x)
        for (int c = 0; c < 3; ++c) {
            const float v = g[3 * i + c];
            if (isfinite(v)) {
                mn[c] = fminf(mn[c], v);
                mx[c] = fmaxf(mx[c], v);
            }
        }
    for (int o = 16; o; o >>= 1)
        for (int c = 0; c < 3; ++c) {
            mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
            mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int c = 0; c < 3; ++c) {
            red[c][warp] = mn[c];
            red[3 + c][warp] = mx[c];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 1; w < nw; ++w)
            for (int c = 0; c < 3; ++c) {
                red[c][0] = fminf(red[c][0], red[c][w]);
                red[3 + c][0] = fmaxf(red[3 + c][0], red[3 + c][w]);
            }
        double ext[3], vol = 1.0, emax = 0.0;
        GridDesc d;
        for (int c = 0; c < 3; ++c) {
            const bool ok = red[c][0] <= red[3 + c][0];
            d.lo[c] = ok ? red[c][0] : 0.f;
            ext[c] = ok ? (double)red[3 + c][0] - (double)red[c][0] : 0.0;
            emax = fmax(emax, ext[c]);
        }
        if (!(emax > 0.0)) emax = 1.0;
        const double target = fmax(1.0, 0.5 * (double)G);
        for (int c = 0; c < 3; ++c) vol *= fmax(ext[c], emax * 1e-3);
        double cell = fmax(cbrt(vol / target), emax / 512.0);
        // every axis covers its extent: [lo, lo + n cell) contains all guides
        for (;;) {
            long long cells = 1;
            bool ok = true;
            for (int c = 0; c < 3; ++c) {
                const double nc = floor(ext[c] / cell) + 1.0;
                ok = ok && nc <= 1024.0;
                d.n[c] = (int)fmin(nc, 1024.0);
                cells *= d.n[c];
            }
            if (ok && cells <= max_cells) break;
            cell *= 1.25;
        }
        d.cell = (float)cell;
        d.inv_cell = (float)(1.0 / cell);
        *gd = d;
    }
}

__device__ __forceinline__ int cell_of(const GridDesc& d, float x, float y, float z) {
    const int cx = min(max(cell_coord(x, d.lo[0], d.inv_cell), 0), d.n[0] - 1);
    const int cy = min(max(cell_coord(y, d.lo[1], d.inv_cell), 0), d.n[1] - 1);
    const int cz = min(max(cell_coord(z, d.lo[2], d.inv_cell), 0), d.n[2] - 1);
    return (cz * d.n[1] + cy) * d.n[0] + cx;
}

__global__ void lbs_cell_count_kernel(int G, const float* __restrict__ g, const GridDesc* __restrict__ gd,
                                      int32_t* __restrict__ cell_of_guide, int32_t* __restrict__ count) {
    const GridDesc d = *gd;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < G; i += gridDim.x * blockDim.x) {
        const int c = cell_of(d, g[3 * i], g[3 * i + 1], g[3 * i + 2]);
        cell_of_guide[i] = c;
        atomicAdd(count + c, 1);
    }
}

// start (exclusive prefix) of each cell from the inclusive scan; fill with a cursor
__global__ void lbs_cell_fill_kernel(int G, const int32_t* __restrict__ cell_of_guide,
                                     const int32_t* __restrict__ incl, const int32_t* __restrict__ count,
                                     int32_t* __restrict__ cursor, int32_t* __restrict__ cell_guides) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < G; i += gridDim.x * blockDim.x) {
        const int c = cell_of_guide[i];
        const int slot = atomicAdd(cursor + c, 1);
        cell_guides[incl[c] - count[c] + slot] = i;
    }
}

struct Best4 {
    float d[4];
    int i[4];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            d[k] = INFINITY;
            i[k] = 0x7fffffff;
        }
    }
    // keep the 4 smallest (d, index) pairs, sorted
    __device__ __forceinline__ void push(float dd, int ii) {
        if (!(dd < d[3] || (dd == d[3] && ii < i[3]))) return;
        int k = 3;
        while (k > 0 && (dd < d[k - 1] || (dd == d[k - 1] && ii < i[k - 1]))) {
            d[k] = d[k - 1];
            i[k] = i[k - 1];
            --k;
        }
        d[k] = dd;
        i[k] = ii;
    }
};

struct BindArgs {
    int64_t Nv;
    const float* x;
    int G;
    const float* g;
    const GridDesc* gd;
    const int32_t* incl;
    const int32_t* count;
    const int32_t* cell_guides;
    float tau;
    int32_t* idx;
    float* w;
    int32_t* guide_count;
};

__global__ void __launch_bounds__(256) lbs_query_kernel(BindArgs a) {
    const GridDesc d = *a.gd;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < a.Nv; v += (int64_t)gridDim.x * blockDim.x) {
        const float qx = a.x[3 * v], qy = a.x[3 * v + 1], qz = a.x[3 * v + 2];
        Best4 B;
        B.init();
        const int c[3] = {cell_coord(qx, d.lo[0], d.inv_cell), cell_coord(qy, d.lo[1], d.inv_cell),
                          cell_coord(qz, d.lo[2], d.inv_cell)};
        const float q[3] = {qx, qy, qz};
        // rings closer than the grid hold no cell
        int r0 = 0;
        for (int k = 0; k < 3; ++k) r0 = max(r0, c[k] < 0 ? -c[k] : (c[k] >= d.n[k] ? c[k] - d.n[k] + 1 : 0));
        const bool finite = isfinite(qx) && isfinite(qy) && isfinite(qz);
        for (int r = r0; finite; ++r) {
            const int i0 = max(c[0] - r, 0), i1 = min(c[0] + r, d.n[0] - 1);
            const int j0 = max(c[1] - r, 0), j1 = min(c[1] + r, d.n[1] - 1);
            const int k0 = max(c[2] - r, 0), k1 = min(c[2] + r, d.n[2] - 1);
            auto visit = [&](int ix, int jy, int kz) {
                const int cell = (kz * d.n[1] + jy) * d.n[0] + ix;
                const int e = a.incl[cell], s = e - a.count[cell];
                for (int p = s; p < e; ++p) {
                    const int gi = a.cell_guides[p];
                    B.push(d2_of(qx, qy, qz, a.g[3 * gi], a.g[3 * gi + 1], a.g[3 * gi + 2]), gi);
                }
            };
            // cells of the grid at Chebyshev distance exactly r from c
            for (int kz = k0; kz <= k1; ++kz)
                for (int jy = j0; jy <= j1; ++jy) {
                    if (abs(kz - c[2]) == r || abs(jy - c[1]) == r) {
                        for (int ix = i0; ix <= i1; ++ix) visit(ix, jy, kz);
                    } else {
                        const int lo_x = c[0] - r, hi_x = c[0] + r;
                        if (lo_x >= 0 && lo_x < d.n[0]) visit(lo_x, jy, kz);
                        if (r > 0 && hi_x >= 0 && hi_x < d.n[0]) visit(hi_x, jy, kz);
                    }
                }
            // done when the searched cube covers the grid, or no unsearched guide can beat the 4th
            bool covers = true;
            float bound = INFINITY;
            for (int k = 0; k < 3; ++k) {
                if (c[k] - r > 0) {
                    covers = false;
                    bound = fminf(bound, q[k] - (d.lo[k] + (float)(c[k] - r) * d.cell));
                }
                if (c[k] + r < d.n[k] - 1) {
                    covers = false;
                    bound = fminf(bound, (d.lo[k] + (float)(c[k] + r + 1) * d.cell) - q[k]);
                }
            }
            if (covers) break;
            // slack for the FP32 rounding of the cell assignment (relative to the coordinate
            // magnitudes involved) and of d^2
            const float mag = fabsf(qx) + fabsf(qy) + fabsf(qz) + fabsf(d.lo[0]) + fabsf(d.lo[1]) + fabsf(d.lo[2]) +
                              (float)(d.n[0] + d.n[1] + d.n[2] + 3) * d.cell;
            const float bnd = fmaxf(bound - 1e-4f * d.cell - 1e-6f * mag, 0.f);
            if (B.d[3] < bnd * bnd * (1.f - 1e-5f)) break;
        }
        // softmax of -d^2 / tau over the found guides (stable: relative to the nearest)
        float e[4], se = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool ok = B.i[k] != 0x7fffffff && isfinite(B.d[k]);
            e[k] = ok ? expf(-__fdiv_rn(__fsub_rn(B.d[k], B.d[0]), a.tau)) : 0.f;
            se = __fadd_rn(se, e[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool ok = B.i[k] != 0x7fffffff && isfinite(B.d[k]);
            a.idx[4 * v + k] = ok ? B.i[k] : -1;
            a.w[4 * v + k] = ok ? __fdiv_rn(e[k], se) : 0.f;
            if (ok) atomicAdd(a.guide_count + B.i[k], 1);
        }
    }
}

__global__ void lbs_inverse_fill_kernel(int64_t Nv, const int32_t* __restrict__ idx, const int32_t* __restrict__ off,
                                        int32_t* __restrict__ cursor, int32_t* __restrict__ ent) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 4 * Nv; e += (int64_t)gridDim.x * blockDim.x) {
        const int k = idx[e];
        if (k < 0) continue;
        const int slot = atomicAdd(cursor + k, 1);
        ent[off[k] + slot] = (int32_t)e;
    }
}

// ascending sort of a[0..len) in place by one CTA: bitonic network in the all-ascending
// ("flip") form, so the virtual +inf padding up to the power of two never moves
__device__ void cta_sort(int32_t* a, int64_t len) {
    int64_t n2 = 1;
    while (n2 < len) n2 <<= 1;
    for (int64_t k = 2; k <= n2; k <<= 1) {
        for (int64_t m = k; m >= 2; m >>= 1) {
            for (int64_t t = threadIdx.x; t < n2 / 2; t += blockDim.x) {
                const int64_t half = m >> 1;
                const int64_t blk = (t / half) * m, off = t % half;
                const int64_t i = blk + off;
                const int64_t j = m == k ? blk + m - 1 - off : i + half;
                if (j < len) {
                    const int32_t x = a[i], y = a[j];
                    if (x > y) {
                        a[i] = y;
                        a[j] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
}

constexpr int kSortSmem = 4096;

__global__ void __launch_bounds__(256) lbs_sort_lists_kernel(int G, const int32_t* __restrict__ off,
                                                              int32_t* __restrict__ ent) {
    __shared__ int32_t buf[kSortSmem];
    for (int k = blockIdx.x; k < G; k += gridDim.x) {
        const int len = off[k + 1] - off[k];
        int32_t* seg = ent + off[k];
        if (len <= 1) continue;
        if (len <= kSortSmem) {
            for (int t = threadIdx.x; t < len; t += blockDim.x) buf[t] = seg[t];
            __syncthreads();
            cta_sort(buf, len);
            for (int t = threadIdx.x; t < len; t += blockDim.x) seg[t] = buf[t];
            __syncthreads();
        } else {
            cta_sort(seg, len);
        }
    }
}

__global__ void __launch_bounds__(256) lbs_forward_kernel(int64_t Nv, const float* __restrict__ x,
                                                          const int4* __restrict__ idx, const float4* __restrict__ w,
                                                          int G, const float4* __restrict__ M, float* __restrict__ y) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < Nv; v += (int64_t)gridDim.x * blockDim.x) {
        const float x0 = x[3 * v], x1 = x[3 * v + 1], x2 = x[3 * v + 2];
        const int4 id = __ldg(idx + v);
        const float4 wv = __ldg(w + v);
        const int ids[4] = {id.x, id.y, id.z, id.w};
        const float ws[4] = {wv.x, wv.y, wv.z, wv.w};
        float o0 = 0.f, o1 = 0.f, o2 = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (ids[k] < 0 || ids[k] >= G) continue;
            const float4* m = M + 3 * (int64_t)ids[k];
            const float4 r0 = __ldg(m), r1 = __ldg(m + 1), r2 = __ldg(m + 2);
            const float y0 = __fmaf_rn(r0.x, x0, __fmaf_rn(r0.y, x1, __fmaf_rn(r0.z, x2, r0.w)));
            const float y1 = __fmaf_rn(r1.x, x0, __fmaf_rn(r1.y, x1, __fmaf_rn(r1.z, x2, r1.w)));
            const float y2 = __fmaf_rn(r2.x, x0, __fmaf_rn(r2.y, x1, __fmaf_rn(r2.z, x2, r2.w)));
            o0 = __fmaf_rn(ws[k], y0, o0);
            o1 = __fmaf_rn(ws[k], y1, o1);
            o2 = __fmaf_rn(ws[k], y2, o2);
        }
        y[3 * v] = o0;
        y[3 * v + 1] = o1;
        y[3 * v + 2] = o2;
    }
}

// dx = sum_k w_k A_k^T gy (weights held fixed, as bound)
__global__ void __launch_bounds__(256) lbs_backward_x_kernel(int64_t Nv, const int4* __restrict__ idx,
                                                             const float4* __restrict__ w, int G,
                                                             const float4* __restrict__ M,
                                                             const float* __restrict__ gy, float* __restrict__ dx) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < Nv; v += (int64_t)gridDim.x * blockDim.x) {
        const float g0 = gy[3 * v], g1 = gy[3 * v + 1], g2 = gy[3 * v + 2];
        const int4 id = __ldg(idx + v);
        const float4 wv = __ldg(w + v);
        const int ids[4] = {id.x, id.y, id.z, id.w};
        const float ws[4] = {wv.x, wv.y, wv.z, wv.w};
        float o0 = 0.f, o1 = 0.f, o2 = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (ids[k] < 0 || ids[k] >= G) continue;
            const float4* m = M + 3 * (int64_t)ids[k];
            const float4 r0 = __ldg(m), r1 = __ldg(m + 1), r2 = __ldg(m + 2);
            const float a0 = __fmaf_rn(r0.x, g0, __fmaf_rn(r1.x, g1, __fmul_rn(r2.x, g2)));
            const float a1 = __fmaf_rn(r0.y, g0, __fmaf_rn(r1.y, g1, __fmul_rn(r2.y, g2)));
            const float a2 = __fmaf_rn(r0.z, g0, __fmaf_rn(r1.z, g1, __fmul_rn(r2.z, g2)));
            o0 = __fmaf_rn(ws[k], a0, o0);
            o1 = __fmaf_rn(ws[k], a1, o1);
            o2 = __fmaf_rn(ws[k], a2, o2);
        }
        dx[3 * v] = o0;
        dx[3 * v + 1] = o1;
        dx[3 * v + 2] = o2;
    }
}

// dM_k = sum over the vertices bound to k of w * gy (x, 1)^T: one warp per guide, entries
// in the sorted order of the bind, fixed lane assignment and reduction tree
__global__ void __launch_bounds__(256) lbs_backward_m_kernel(int G, const int32_t* __restrict__ off,
                                                             const int32_t* __restrict__ ent,
                                                             const float* __restrict__ x, const float* __restrict__ w,
                                                             const float* __restrict__ gy, float* __restrict__ dM) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t k = warp0; k < G; k += nw) {
        const int e0 = off[k], e1 = off[k + 1];
        float acc[12];
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = 0.f;
        for (int p = e0 + lane; p < e1; p += 32) {
            const int e = __ldg(ent + p);
            const int64_t v = e >> 2;
            const float wv = __ldg(w + e);
            const float xh[4] = {__ldg(x + 3 * v), __ldg(x + 3 * v + 1), __ldg(x + 3 * v + 2), 1.f};
            const float gw[3] = {__fmul_rn(wv, __ldg(gy + 3 * v)), __fmul_rn(wv, __ldg(gy + 3 * v + 1)),
                                 __fmul_rn(wv, __ldg(gy + 3 * v + 2))};
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[4 * r + c] = __fmaf_rn(gw[r], xh[c], acc[4 * r + c]);
        }
#pragma unroll
        for (int q = 0; q < 12; ++q)
#pragma unroll
            for (int o = 16; o; o >>= 1) acc[q] = __fadd_rn(acc[q], __shfl_xor_sync(0xffffffffu, acc[q], o));
        if (lane < 12) {
            float val = acc[0];
#pragma unroll
            for (int q = 1; q < 12; ++q)
                if (lane == q) val = acc[q];
            dM[12 * k + lane] = val;
        }
    }
}

struct BindWs {
    GridDesc* gd;
    int cells;
    int32_t *cell_count, *cell_incl, *cell_cursor, *cell_guides, *cell_of_guide, *guide_cursor;
    int64_t* total;
    void* scan_ws;
};

int cells_cap(int G) { return (int)std::min<int64_t>(kMaxCells, 2 * (int64_t)G + 1024); }

size_t bind_carve(int G, void* base, size_t cap, BindWs* w) {
    Carver cv(base, cap);
    BindWs t;
    t.cells = cells_cap(G);
    t.gd = cv.take<GridDesc>(1);
    t.total = cv.take<int64_t>(1);
    t.cell_count = cv.take<int32_t>(t.cells);
    t.cell_incl = cv.take<int32_t>(t.cells);
    t.cell_cursor = cv.take<int32_t>(t.cells);
    t.cell_guides = cv.take<int32_t>(std::max(G, 1));
    t.cell_of_guide = cv.take<int32_t>(std::max(G, 1));
    t.guide_cursor = cv.take<int32_t>(std::max(G, 1));
    t.scan_ws = cv.take<char>(scan_workspace_bytes(std::max(t.cells, G)));
    if (w) *w = t;
    return cv.off;
}

}  // namespace
}  // namespace s2c

using namespace s2c;

extern "C" {

S2C_API s2c_status s2c_card_laplacian_smooth(int num_cards, int verts_per_card, const int32_t* adj_offsets,
                                             const int32_t* adj, int num_adj, const float* verts_in,
                                             float* verts_out, float lam, int steps, s2c_stream stream) {
    S2C_REQUIRE(num_cards >= 0 && verts_per_card >= 0 && num_adj >= 0 && steps >= 0,
                "card_laplacian_smooth: negative size");
    if (num_cards == 0 || verts_per_card == 0) return S2C_OK;
    S2C_REQUIRE(adj_offsets && verts_in && verts_out && (num_adj == 0 || adj), "card_laplacian_smooth: null pointer");
    const int nv = verts_per_card;
    const size_t topo = (size_t)(nv + 1 + num_adj) * 4;
    const size_t per_card = (size_t)nv * 24;
    S2C_REQUIRE(topo + per_card <= (size_t)kLapSmem,
                "card_laplacian_smooth: a card of %d vertices and %d adjacency entries exceeds shared memory", nv,
                num_adj);
    LapArgs a;
    a.num_cards = num_cards;
    a.nv = nv;
    // cards per CTA: fill the threads, within the shared-memory budget
    const int fit = (int)((kLapSmem - topo) / per_card);
    a.cpc = std::max(1, std::min(fit, (kLapThreads * 2 + nv - 1) / nv));
    a.ngroups = (num_cards + a.cpc - 1) / a.cpc;
    a.nadj = num_adj;
    a.steps = steps;
    a.off = adj_offsets;
    a.adj = adj;
    a.in = verts_in;
    a.out = verts_out;
    a.lam = lam;
    const size_t smem = topo + (size_t)a.cpc * per_card;
    const int blocks = (int)std::min<int64_t>(a.ngroups, (int64_t)num_sms() * 8);
    card_laplacian_kernel<<<blocks, kLapThreads, smem, (cudaStream_t)stream>>>(a);
    S2C_CHECK_LAUNCH("card_laplacian_kernel");
    return S2C_OK;
}

S2C_API size_t s2c_lbs_bind_workspace_size(int64_t num_verts, int num_guides) {
    (void)num_verts;
    return bind_carve(num_guides, nullptr, (size_t)-1, nullptr) + 256;
}

S2C_API s2c_status s2c_lbs_bind(int64_t Nv, const float* x, int G, const float* guides, float tau, int32_t* idx,
                                float* w, int32_t* list_offsets, int32_t* list_entries, void* workspace,
                                size_t workspace_bytes, s2c_stream stream) {
    S2C_REQUIRE(Nv >= 0 && G >= 0, "lbs_bind: negative size");
    S2C_REQUIRE(4 * Nv < (1LL << 31), "lbs_bind: too many vertices (%lld)", (long long)Nv);
    S2C_REQUIRE(tau > 0.f, "lbs_bind: tau must be positive");
    S2C_REQUIRE(list_offsets && (G == 0 || guides) && (Nv == 0 || (x && idx && w && list_entries)),
                "lbs_bind: null pointer");
    S2C_REQUIRE(((uintptr_t)idx & 15) == 0 && ((uintptr_t)w & 15) == 0, "lbs_bind: idx / w not 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    if (G == 0) {
        if (Nv > 0) {
            cudaError_t e = cudaMemsetAsync(idx, 0xff, (size_t)Nv * 16, st);
            if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, (size_t)Nv * 16, st);
            if (e != cudaSuccess) return cuda_status(e, "lbs_bind: memset");
        }
        return S2C_OK;
    }
    BindWs B;
    const size_t need = bind_carve(G, workspace, workspace_bytes, &B);
    S2C_REQUIRE(workspace && need <= workspace_bytes, "lbs_bind: workspace of %zu bytes, need %zu", workspace_bytes,
                need);
    cudaError_t e = cudaMemsetAsync(B.cell_count, 0, sizeof(int32_t) * B.cells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.cell_cursor, 0, sizeof(int32_t) * B.cells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.guide_cursor, 0, sizeof(int32_t) * G, st);
    if (e != cudaSuccess) return cuda_status(e, "lbs_bind: memset");
    lbs_grid_kernel<<<1, 1024, 0, st>>>(G, guides, B.cells, B.gd);
    S2C_CHECK_LAUNCH("lbs_grid_kernel");
    const unsigned gb = grid_for(G, 256, (int64_t)num_sms() * 8);
    lbs_cell_count_kernel<<<gb, 256, 0, st>>>(G, guides, B.gd, B.cell_of_guide, B.cell_count);
    S2C_CHECK_LAUNCH("lbs_cell_count_kernel");
    s2c_status s = inclusive_scan_i32(B.cell_count, B.cells, B.cell_incl, B.scan_ws, B.total, st);
    if (s != S2C_OK) return s;
    lbs_cell_fill_kernel<<<gb, 256, 0, st>>>(G, B.cell_of_guide, B.cell_incl, B.cell_count, B.cell_cursor,
                                             B.cell_guides);
    S2C_CHECK_LAUNCH("lbs_cell_fill_kernel");
    if (Nv == 0) return S2C_OK;
    // per-guide vertex counts, in cell_of_guide (no longer needed after the fill)
    int32_t* gcount = B.cell_of_guide;
    e = cudaMemsetAsync(gcount, 0, sizeof(int32_t) * G, st);
    if (e != cudaSuccess) return cuda_status(e, "lbs_bind: memset");
    BindArgs a;
    a.Nv = Nv;
    a.x = x;
    a.G = G;
    a.g = guides;
    a.gd = B.gd;
    a.incl = B.cell_incl;
    a.count = B.cell_count;
    a.cell_guides = B.cell_guides;
    a.tau = tau;
    a.idx = idx;
    a.w = w;
    a.guide_count = gcount;
    lbs_query_kernel<<<grid_for(Nv, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(a);
    S2C_CHECK_LAUNCH("lbs_query_kernel");
    // list_offsets (G + 1): 0, then the inclusive prefix of the per-guide counts
    e = cudaMemsetAsync(list_offsets, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return cuda_status(e, "lbs_bind: memset");
    s = inclusive_scan_i32(gcount, G, list_offsets + 1, B.scan_ws, B.total, st);
    if (s != S2C_OK) return s;
    lbs_inverse_fill_kernel<<<grid_for(4 * Nv, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(
        Nv, idx, list_offsets, B.guide_cursor, list_entries);
    S2C_CHECK_LAUNCH("lbs_inverse_fill_kernel");
    lbs_sort_lists_kernel<<<(unsigned)std::min<int64_t>(G, (int64_t)num_sms() * 16), 256, 0, st>>>(
        G, list_offsets, list_entries);
    S2C_CHECK_LAUNCH("lbs_sort_lists_kernel");
    return S2C_OK;
}

S2C_API s2c_status s2c_lbs_forward(int64_t Nv, const float* x, const int32_t* idx, const float* w, int G,
                                   const float* M, float* y, s2c_stream stream) {
    S2C_REQUIRE(Nv >= 0 && G >= 0, "lbs_forward: negative size");
    if (Nv == 0) return S2C_OK;
    S2C_REQUIRE(x && idx && w && y && (G == 0 || M), "lbs_forward: null pointer");
    S2C_REQUIRE(((uintptr_t)idx & 15) == 0 && ((uintptr_t)w & 15) == 0 && ((uintptr_t)M & 15) == 0,
                "lbs_forward: idx / w / M not 16-byte aligned");
    lbs_forward_kernel<<<grid_for(Nv, 256, (int64_t)num_sms() * 16), 256, 0, (cudaStream_t)stream>>>(
        Nv, x, (const int4*)idx, (const float4*)w, G, (const float4*)M, y);
    S2C_CHECK_LAUNCH("lbs_forward_kernel");
    return S2C_OK;
}

S2C_API s2c_status s2c_lbs_backward(int64_t Nv, const float* x, const int32_t* idx, const float* w, int G,
                                    const float* M, const int32_t* list_offsets, const int32_t* list_entries,
                                    const float* grad_y, float* grad_M, float* grad_x, s2c_stream stream) {
    S2C_REQUIRE(Nv >= 0 && G >= 0, "lbs_backward: negative size");
    cudaStream_t st = (cudaStream_t)stream;
    if (grad_M && G > 0) {
        S2C_REQUIRE(list_offsets && (Nv == 0 || (list_entries && x && w && grad_y)), "lbs_backward: null pointer");
        if (Nv == 0) {
            cudaError_t e = cudaMemsetAsync(grad_M, 0, (size_t)G * 48, st);
            if (e != cudaSuccess) return cuda_status(e, "lbs_backward: memset");
        } else {
            lbs_backward_m_kernel<<<grid_for((int64_t)G * 32, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(
                G, list_offsets, list_entries, x, w, grad_y, grad_M);
            S2C_CHECK_LAUNCH("lbs_backward_m_kernel");
        }
    }
    if (grad_x && Nv > 0) {
        S2C_REQUIRE(idx && w && grad_y && (G == 0 || M), "lbs_backward: null pointer");
        S2C_REQUIRE(((uintptr_t)idx & 15) == 0 && ((uintptr_t)w & 15) == 0 && ((uintptr_t)M & 15) == 0,
                    "lbs_backward: idx / w / M not 16-byte aligned");
        lbs_backward_x_kernel<<<grid_for(Nv, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(
            Nv, (const int4*)idx, (const float4*)w, G, (const float4*)M, grad_y, grad_x);
        S2C_CHECK_LAUNCH("lbs_backward_x_kernel");
    }
    return S2C_OK;
}

}  // extern "C"
