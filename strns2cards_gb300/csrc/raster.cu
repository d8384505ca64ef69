// Triangle rasterisation, depth test and attribute interpolation (the reference's
// rasterize.cu:9-472 and dda.cu:258-342), entry for entry, with the same FP32 arithmetic:
// coverage, barycentrics, depth and triangle ids are bit-identical to the reference.
//
// Depth test: the reference keeps, per pixel, the minimum of (bits(z + 2) << 32 | fragment
// index) with a 64-bit atomicMin (rasterize.cu:198-229); the fragment index there is the
// position after a compaction whose order depends on block scheduling.  Here the
// compaction keeps input order, so exact depth ties resolve to the first fragment in
// (view, triangle, row-major pixel) order, deterministically.
#include <algorithm>
#include <climits>

#include "common.cuh"
#include "scan.cuh"
#include "list.cuh"
#include "tri.cuh"

namespace s2c {

struct Tris {
    const float4* __restrict__ pos4;  // (B, V)
    const int* __restrict__ tri;      // (T, 3)
    int V, T;
    FastDiv divT;
};

// rasterize.cu:9-59: screen rectangle (h0, h_len, w0, w_len) of triangle (b, t)
__device__ __forceinline__ int4 tri_rect(int H, int W, const Tris& R, int b, int t) {
    float4 P[3];
    bool ok[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int v = __ldg(R.tri + 3 * t + i);
        ok[i] = (unsigned)v < (unsigned)R.V;
        P[i] = ok[i] ? __ldg(R.pos4 + (int64_t)b * R.V + v) : make_float4(0.f, 0.f, 0.f, 1.f);
    }
    return tri_rect_of(H, W, P, ok);
}

__global__ void __launch_bounds__(256) tri_rects_kernel(int H, int W, int B, Tris R, int4* __restrict__ rects,
                                                        int32_t* __restrict__ counts) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * R.T) return;
    const int b = (int)R.divT.div((uint32_t)idx);
    const int t = (int)idx - b * R.T;
    const int4 rc = tri_rect(H, W, R, b, t);
    rects[idx] = rc;
    counts[idx] = (int32_t)((uint32_t)rc.y * (uint32_t)rc.w);
}

// rasterize.cu:90-172: one thread per bounding-box pixel, owner triangle by binary search
__global__ void __launch_bounds__(256) tri_fragments_kernel(int H, int W, Tris R, int64_t BT, int64_t F,
                                                            const int32_t* __restrict__ prefix,
                                                            const int4* __restrict__ rects,
                                                            int32_t* __restrict__ frag_pix,
                                                            float4* __restrict__ frag_attrs) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= F) return;
    int64_t lo = 0, hi = BT;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)(uint32_t)__ldg(prefix + mid) <= idx) lo = mid + 1;
        else hi = mid;
    }
    if (lo >= BT) return;
    const int b = (int)R.divT.div((uint32_t)lo);
    const int t = (int)lo - b * R.T;
    const int4 rc = __ldg(rects + lo);
    if (rc.w <= 0 || rc.y <= 0) return;
    const int local = (int)(idx - (lo ? (int64_t)(uint32_t)__ldg(prefix + lo - 1) : 0));
    const int y = rc.x + local / rc.w;
    const int x = rc.z + local % rc.w;
    if (x < 0 || x >= W || y < 0 || y >= H) return;
    const int i0 = __ldg(R.tri + 3 * t), i1 = __ldg(R.tri + 3 * t + 1), i2 = __ldg(R.tri + 3 * t + 2);
    if ((unsigned)i0 >= (unsigned)R.V || (unsigned)i1 >= (unsigned)R.V || (unsigned)i2 >= (unsigned)R.V) return;
    const float4* pb = R.pos4 + (int64_t)b * R.V;
    float b0, b1, z;
    if (!tri_cover(H, W, __ldg(pb + i0), __ldg(pb + i1), __ldg(pb + i2), x, y, b0, b1, z)) return;
    frag_pix[3 * idx] = b;
    frag_pix[3 * idx + 1] = y;
    frag_pix[3 * idx + 2] = x;
    frag_attrs[idx] = make_float4(b0, b1, z, (float)(t + 1));
}

// keys are stored as (signed key) ^ 2^63 so that unsigned atomicMin orders them like the
// reference's signed long long; the empty value LLONG_MAX maps to all ones
__global__ void fill_keys(unsigned long long* __restrict__ keys, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = 0xffffffffffffffffull;
}

// rasterize.cu:209-229 (keys compared as signed 64-bit, as the reference's long long;
// z + 2 > 0 for every accepted fragment, so the unsigned compare orders them the same)
__global__ void __launch_bounds__(256) depth_keys_kernel(int64_t F, const int32_t* __restrict__ frag_pix,
                                                         const float4* __restrict__ frag_attrs, int B, int H, int W,
                                                         unsigned long long* __restrict__ keys) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F) return;
    const int b = frag_pix[3 * i], h = frag_pix[3 * i + 1], w = frag_pix[3 * i + 2];
    if (b < 0 || b >= B || h < 0 || h >= H || w < 0 || w >= W) return;
    const float zz = __fadd_rn(frag_attrs[i].z, 2.f);
    // the reference's signed key (bits(z + 2) << 32) | index, as a bit pattern, mapped to an
    // order-preserving unsigned value
    const unsigned long long key = ((unsigned long long)(uint32_t)__float_as_int(zz) << 32) | (uint32_t)i;
    const unsigned long long ukey = key ^ 0x8000000000000000ull;
    atomicMin(keys + ((int64_t)b * H + h) * W + w, ukey);
}

__global__ void __launch_bounds__(256) depth_gather_kernel(int64_t npix, const unsigned long long* __restrict__ keys,
                                                           const float4* __restrict__ frag_attrs, int64_t F,
                                                           float4* __restrict__ rast) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const unsigned long long k = keys[p] ^ 0x8000000000000000ull;
    if (k == 0xffffffffffffffffull) return;  // no fragment (the fill value)
    const int fi = (int)(uint32_t)(k & 0xffffffffull);
    if (fi < 0 || fi >= F) return;
    rast[p] = frag_attrs[fi];
}

// Fused raster (compute_fragments + depth_test + cluster_mask_from_fragments without the
// fragment list).  A covered pixel ORs its cluster bit into the bitset and offers the key
// (bits(z + 2) << 32 | t) to the pixel's 64-bit minimum: within one pixel the list path's
// fragment order is triangle order, so the minimum picks the fragment the list-based
// depth test picks.
struct FusedRaster {
    int B, H, W, S;
    Tris R;
    const int32_t* __restrict__ t2c;        // nullable
    int num_t2c;
    int32_t* __restrict__ bitset;           // nullable
    uint32_t* __restrict__ planes;          // nullable: cluster planes (B, 32 S, H, WQ)
    int WQ;
    unsigned long long* __restrict__ keys;  // nullable
    const int4* __restrict__ rects;         // (B*T) screen rectangles
    const uint32_t* __restrict__ prefix;    // (B*T) inclusive prefix of their areas
    const int64_t* __restrict__ total;      // device: sum of the areas
};

// one pixel of a triangle whose corners are loaded
__device__ __forceinline__ void raster_covered(const FusedRaster& F, const float* px_lut, const float* py_lut, int ob,
                                               int ot, float4 P0, float4 P1, float4 P2, int x, int y) {
    if (x < 0 || x >= F.W || y < 0 || y >= F.H) return;
    const float px = px_lut ? px_lut[x] : ndc_of(x, (float)F.W);
    const float py = py_lut ? py_lut[y] : ndc_of(y, (float)F.H);
    const TriEdges e = tri_edges(P0, P1, P2, px, py);
    if (tri_surely_outside(e)) return;
    float b0, b1, z;
    if (!tri_finish(e, P0, P1, P2, b0, b1, z)) return;
    const int64_t pix = ((int64_t)ob * F.H + y) * F.W + x;
    if (F.keys) {
        const float zz = __fadd_rn(z, 2.f);
        atomicMin(F.keys + pix, ((unsigned long long)(uint32_t)__float_as_int(zz) << 32) | (uint32_t)ot);
    }
    if ((F.bitset || F.planes) && ot < F.num_t2c) {
        const int c = __ldg(F.t2c + ot);
        if (c >= 0 && c < 32 * F.S) {
            if (F.bitset) atomicOr(F.bitset + pix * F.S + (c >> 5), (int32_t)(1u << (c & 31)));
            if (F.planes)
                atomicOr(F.planes + (((int64_t)ob * 32 * F.S + c) * F.H + y) * F.WQ + (x >> 5), 1u << (x & 31));
        }
    }
}

// the corners of triangle ot of view ob; false for an out-of-range vertex index
__device__ __forceinline__ bool raster_corners(const FusedRaster& F, int ob, int ot, float4& P0, float4& P1,
                                               float4& P2) {
    const int i0 = __ldg(F.R.tri + 3 * ot), i1 = __ldg(F.R.tri + 3 * ot + 1), i2 = __ldg(F.R.tri + 3 * ot + 2);
    if ((unsigned)i0 >= (unsigned)F.R.V || (unsigned)i1 >= (unsigned)F.R.V || (unsigned)i2 >= (unsigned)F.R.V)
        return false;
    const float4* pb = F.R.pos4 + (int64_t)ob * F.R.V;
    P0 = __ldg(pb + i0);
    P1 = __ldg(pb + i1);
    P2 = __ldg(pb + i2);
    return true;
}

__device__ __forceinline__ void raster_pixel(const FusedRaster& F, const float* px_lut, const float* py_lut, int ob,
                                             int ot, int x, int y) {
    if (x < 0 || x >= F.W || y < 0 || y >= F.H) return;
    float4 P0, P1, P2;
    if (!raster_corners(F, ob, ot, P0, P1, P2)) return;
    raster_covered(F, px_lut, py_lut, ob, ot, P0, P1, P2, x, y);
}

// local / w for 0 <= local, 1 <= w: float estimate corrected by one step (exact while
// local < 2^22), integer division beyond
__device__ __forceinline__ int divmod_small(int local, int w, int& r) {
    int q;
    if (local < (1 << 22)) {
        q = __float2int_rz(__fmul_rn(__int2float_rn(local), __frcp_rn((float)w)));
        r = local - q * w;
        if (r < 0) { --q; r += w; }
        else if (r >= w) { ++q; r -= w; }
    } else {
        q = local / w;
        r = local - q * w;
    }
    return q;
}

// The compacted fragment list (what filter_valid_fragments leaves of tri_fragments_kernel's
// list) in two passes over the same bounding-box pixel index space (list.cuh).
template <bool kWrite>
__global__ void __launch_bounds__(256) tri_list_kernel(int H, int W, Tris R, int64_t BT, uint32_t F,
                                                       const int32_t* __restrict__ prefix,
                                                       const int4* __restrict__ rects, uint32_t* __restrict__ mask,
                                                       const int32_t* __restrict__ wpre, int32_t* __restrict__ frag_pix,
                                                       float4* __restrict__ frag_attrs) {
    // pixel k of triangle o's box, covered: (b, y, x) and (b0, b1, z)
    auto cover = [&](int64_t o, int k, int& b, int& t, int& x, int& y, float& b0, float& b1, float& z) {
        b = (int)R.divT.div((uint32_t)o);
        t = (int)o - b * R.T;
        const int4 rc = __ldg(rects + o);
        if (rc.w <= 0 || rc.y <= 0) return false;
        int r;
        const int q = divmod_small(k, rc.w, r);
        y = rc.x + q;
        x = rc.z + r;
        if (x < 0 || x >= W || y < 0 || y >= H) return false;
        const int i0 = __ldg(R.tri + 3 * t), i1 = __ldg(R.tri + 3 * t + 1), i2 = __ldg(R.tri + 3 * t + 2);
        if ((unsigned)i0 >= (unsigned)R.V || (unsigned)i1 >= (unsigned)R.V || (unsigned)i2 >= (unsigned)R.V)
            return false;
        const float4* pb = R.pos4 + (int64_t)b * R.V;
        return tri_cover(H, W, __ldg(pb + i0), __ldg(pb + i1), __ldg(pb + i2), x, y, b0, b1, z);
    };
    list_pass<kWrite>(
        BT, F, prefix, mask, wpre,
        [&](int64_t o, int k) {
            int b, t, x, y;
            float b0, b1, z;
            return cover(o, k, b, t, x, y, b0, b1, z);
        },
        [&](int64_t o, int k, int64_t at) {
            int b = 0, t = 0, x = 0, y = 0;
            float b0 = 0.f, b1 = 0.f, z = 0.f;
            cover(o, k, b, t, x, y, b0, b1, z);   // accepted in pass 1: the same values again
            frag_pix[3 * at] = b;
            frag_pix[3 * at + 1] = y;
            frag_pix[3 * at + 2] = x;
            frag_attrs[at] = make_float4(b0, b1, z, (float)(t + 1));
        });
}


constexpr int kRasterChunk = 1024;
// pixels of one bounding-box row per work unit (the triangle's corners loaded once for all):
// 2 -> 4 took the config-2 card raster from 0.388 to 0.367 ms; 8 was slower (0.419 ms: the
// thin cards' boxes leave more of each run outside)
constexpr int kRasterRun = 4;

// Balanced pass: warps take equal chunks of the global bbox-pixel index space.  A warp
// keeps a window of 32 consecutive triangles' prefix values in its lanes, slides it along
// the chunk, and each lane finds the owner of its pixel with a 5-step shuffle search.
__global__ void __launch_bounds__(256, 4) tri_fused_kernel(FusedRaster F) {
    extern __shared__ float lut[];
    const bool use_lut = F.W + F.H <= 8192;
    if (use_lut) {
        for (int i = threadIdx.x; i < F.W; i += blockDim.x) lut[i] = ndc_of(i, (float)F.W);
        for (int i = threadIdx.x; i < F.H; i += blockDim.x) lut[F.W + i] = ndc_of(i, (float)F.H);
        __syncthreads();
    }
    const float* px_lut = use_lut ? lut : nullptr;
    const float* py_lut = use_lut ? lut + F.W : nullptr;
    const int lane = threadIdx.x & 31;
    const int64_t BT = (int64_t)F.B * F.R.T;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t total = *F.total;
    if (total > 0xffffffffLL) {
        // areas beyond 32 bits: each warp walks 32 whole triangles (correct, unbalanced)
        for (int64_t g = warp0 * 32; g < BT; g += nwarps * 32) {
            const int64_t mine = g + lane;
            int4 rc = make_int4(0, 0, 0, 0);
            int b = 0, t = 0;
            if (mine < BT) {
                b = (int)F.R.divT.div((uint32_t)mine);
                t = (int)mine - b * F.R.T;
                rc = F.rects[mine];
            }
            for (int k = 0; k < rc.y * rc.w; ++k) {
                int r;
                const int q = divmod_small(k, rc.w, r);
                raster_pixel(F, px_lut, py_lut, b, t, rc.z + r, rc.x + q);
            }
        }
        return;
    }
    const uint32_t tot = (uint32_t)total;
    const int64_t nchunks = ((int64_t)tot + kRasterChunk - 1) / kRasterChunk;
    for (int64_t ch = warp0; ch < nchunks; ch += nwarps) {
        const uint32_t c0 = (uint32_t)(ch * kRasterChunk);
        const uint32_t c1 = (uint32_t)min((int64_t)tot, (ch + 1) * kRasterChunk);
        // first triangle whose inclusive prefix exceeds c0 (same search on every lane)
        int64_t lo = 0, hi = BT;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (__ldg(F.prefix + mid) <= c0) lo = mid + 1;
            else hi = mid;
        }
        int64_t t0 = lo;
        uint32_t start = t0 > 0 ? __ldg(F.prefix + t0 - 1) : 0u;
        uint32_t pre = t0 + lane < BT ? __ldg(F.prefix + t0 + lane) : 0xffffffffu;
        uint32_t base = c0;
        while (base < c1) {
            // slide the window until its first triangle holds `base`
            for (;;) {
                const unsigned m = __ballot_sync(0xffffffffu, pre <= base);
                if (!m) break;
                const int adv = __popc(m);
                start = __shfl_sync(0xffffffffu, pre, adv - 1);
                t0 += adv;
                pre = t0 + lane < BT ? __ldg(F.prefix + t0 + lane) : 0xffffffffu;
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
            if (j < end) {
                // work unit j: a run of kRasterRun horizontally adjacent bounding-box pixels
                // (the triangle's corners are loaded once for all of them)
                const int64_t o = t0 + ow;
                const int ob = (int)F.R.divT.div((uint32_t)o);
                const int ot = (int)o - ob * F.R.T;
                const int4 rc = F.rects[o];
                const int local = (int)(j - (ow > 0 ? prev : start));
                const int wp = (rc.w + (kRasterRun - 1)) / kRasterRun;
                int r;
                const int q = divmod_small(local, wp, r);
                const int x = rc.z + kRasterRun * r, y = rc.x + q;
                float4 P0, P1, P2;
                // only the bounding box's own pixels, as the list path tests
                if (q < rc.y && y >= 0 && y < F.H && raster_corners(F, ob, ot, P0, P1, P2)) {
#pragma unroll
                    for (int u = 0; u < kRasterRun; ++u)
                        if (kRasterRun * r + u < rc.w) raster_covered(F, px_lut, py_lut, ob, ot, P0, P1, P2, x + u, y);
                }
            }
            base = end;
        }
    }
}

// screen rectangle and area of every (view, triangle)
// Per (view, cluster plane) word rectangles (y0, y1, q0, q1): rows [y0, y1) and plane
// words [q0, q1) holding every bit the raster can set (the union of the cluster's triangle
// rectangles); empty = (H, 0, WQ, 0).
struct ClusterRects {
    int4* __restrict__ r;                  // nullable: (B, Kp)
    const int32_t* __restrict__ t2c;
    int num_t2c, Kp;
};

__global__ void cluster_rects_init_kernel(int64_t n, int H, int WQ, int4* __restrict__ r) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = make_int4(H, 0, WQ, 0);
}

__global__ void __launch_bounds__(256) tri_rect_area_kernel(int H, int W, int B, Tris R, int4* __restrict__ rects,
                                                            int32_t* __restrict__ areas, ClusterRects CR) {
    const int64_t n = (int64_t)B * R.T;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)R.divT.div((uint32_t)idx);
        const int t = (int)idx - b * R.T;
        const int4 rc = tri_rect(H, W, R, b, t);
        rects[idx] = rc;
        // work units of the balanced raster: runs of kRasterRun horizontally adjacent pixels
        areas[idx] = (int32_t)((uint32_t)rc.y * (((uint32_t)rc.w + (kRasterRun - 1)) / kRasterRun));
        if (CR.r) {
            // the raster's cluster bit for t (raster_covered); lanes of one (view, cluster) --
            // consecutive triangles of a card -- reduce their rectangles first, and one lane
            // per group extends the cluster's rectangle (a card's 128 triangles would
            // otherwise queue 128 deep on the same four words)
            int64_t key = -1;
            int y0 = INT_MAX, y1 = INT_MIN, q0 = INT_MAX, q1 = INT_MIN;
            if (rc.y > 0 && rc.w > 0 && t < CR.num_t2c) {
                const int c = __ldg(CR.t2c + t);
                if (c >= 0 && c < CR.Kp) {
                    key = (int64_t)b * CR.Kp + c;
                    y0 = rc.x;
                    y1 = rc.x + rc.y;
                    q0 = rc.z >> 5;
                    q1 = ((rc.z + rc.w - 1) >> 5) + 1;
                }
            }
            const unsigned grp = __match_any_sync(__activemask(), key);
            y0 = __reduce_min_sync(grp, y0);
            y1 = __reduce_max_sync(grp, y1);
            q0 = __reduce_min_sync(grp, q0);
            q1 = __reduce_max_sync(grp, q1);
            if (key >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) {
                int* q = (int*)(CR.r + key);
                atomicMin(q + 0, y0);
                atomicMax(q + 1, y1);
                atomicMin(q + 2, q0);
                atomicMax(q + 3, q1);
            }
        }
    }
}

// rast of the winning triangle of every pixel, recomputed with the forward's arithmetic
__global__ void __launch_bounds__(256) tri_resolve_kernel(int B, int H, int W, Tris R,
                                                          const unsigned long long* __restrict__ keys,
                                                          float4* __restrict__ rast) {
    const int64_t n = (int64_t)B * H * W;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[p];
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k != 0xffffffffffffffffull) {
            const int t = (int)(uint32_t)(k & 0xffffffffull);
            const int64_t bh = p / W;
            const int x = (int)(p - bh * W);
            const int b = (int)(bh / H);
            const int y = (int)(bh - (int64_t)b * H);
            const int i0 = __ldg(R.tri + 3 * t), i1 = __ldg(R.tri + 3 * t + 1), i2 = __ldg(R.tri + 3 * t + 2);
            const float4* pb = R.pos4 + (int64_t)b * R.V;
            float b0, b1, z;
            if (tri_cover(H, W, __ldg(pb + i0), __ldg(pb + i1), __ldg(pb + i2), x, y, b0, b1, z))
                o = make_float4(b0, b1, z, (float)(t + 1));
        }
        rast[p] = o;
    }
}

// rasterize.cu:367-400
__global__ void __launch_bounds__(256) interp_kernel(int64_t npix, const float4* __restrict__ rast, int C,
                                                     const float* __restrict__ attr, int V,
                                                     const int* __restrict__ tri, int T, float* __restrict__ image) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float4 r = rast[p];
    const int t = f2i(r.w) - 1;
    if (t < 0 || t >= T) return;
    const float b0 = r.x, b1 = r.y, b2 = __fsub_rn(__fsub_rn(1.f, b0), b1);
    const int v0 = __ldg(tri + 3 * t), v1 = __ldg(tri + 3 * t + 1), v2 = __ldg(tri + 3 * t + 2);
    if ((unsigned)v0 >= (unsigned)V || (unsigned)v1 >= (unsigned)V || (unsigned)v2 >= (unsigned)V) return;
    const float* a0 = attr + (int64_t)C * v0;
    const float* a1 = attr + (int64_t)C * v1;
    const float* a2 = attr + (int64_t)C * v2;
    for (int d = 0; d < C; ++d)
        image[p * C + d] = __fmaf_rn(b2, __ldg(a2 + d), __fmaf_rn(b1, __ldg(a1 + d), __fmul_rn(b0, __ldg(a0 + d))));
}

// Software MSAA resolve (the sample loop of the reference's texture render,
// texture_utils.py:189-226, with interpolate_triangle_attributes folded in): per pixel and
// sample i in order, rgb_i = the interpolated attribute of rast_i (0 where empty), a_i =
// (rast_i.w > 0), acc += rgb_i * a_i, count += a_i, alpha += w_i * a_i -- the FP32 torch
// operations of the reference's loop in the same order, so the sums are identical.
constexpr int kMsaaMaxC = 8;

__global__ void __launch_bounds__(256) msaa_resolve_kernel(int S, int64_t npix, int C, const float4* __restrict__ rast,
                                                           const float* __restrict__ attr, int V,
                                                           const int* __restrict__ tri, int T,
                                                           const float* __restrict__ wts, float* __restrict__ acc,
                                                           float* __restrict__ cnt, float* __restrict__ alpha) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
        float a[kMsaaMaxC];
#pragma unroll
        for (int d = 0; d < kMsaaMaxC; ++d) a[d] = 0.f;
        float n = 0.f, al = 0.f;
        for (int i = 0; i < S; ++i) {
            const float4 r = __ldcs(rast + (int64_t)i * npix + p);
            const float av = r.w > 0.f ? 1.f : 0.f;
            const int t = f2i(r.w) - 1;
            bool ok = t >= 0 && t < T;
            int v0 = 0, v1 = 0, v2 = 0;
            if (ok) {
                v0 = __ldg(tri + 3 * t);
                v1 = __ldg(tri + 3 * t + 1);
                v2 = __ldg(tri + 3 * t + 2);
                ok = (unsigned)v0 < (unsigned)V && (unsigned)v1 < (unsigned)V && (unsigned)v2 < (unsigned)V;
            }
            const float b0 = r.x, b1 = r.y, b2 = __fsub_rn(__fsub_rn(1.f, b0), b1);
#pragma unroll
            for (int d = 0; d < kMsaaMaxC; ++d) {
                if (d >= C) break;
                float rgb = 0.f;
                if (ok)
                    rgb = __fmaf_rn(b2, __ldg(attr + (int64_t)C * v2 + d),
                                    __fmaf_rn(b1, __ldg(attr + (int64_t)C * v1 + d),
                                              __fmul_rn(b0, __ldg(attr + (int64_t)C * v0 + d))));
                a[d] = __fadd_rn(a[d], __fmul_rn(rgb, av));
            }
            n = __fadd_rn(n, av);
            al = __fadd_rn(al, __fmul_rn(__ldg(wts + i), av));
        }
        for (int d = 0; d < C; ++d) acc[p * C + d] = a[d];
        cnt[p] = n;
        alpha[p] = al;
    }
}

// rasterize.cu:402-438: scatter-add of grad * b_i.  Acc = float: float atomics into d_attr,
// as the reference.  Acc = double: each FP32 x FP32 product is exact in FP64 and is summed
// there (FP64 L2 atomics into a caller accumulator); finish_acc64 rounds each sum once.
template <typename Acc>
__device__ __forceinline__ void acc_add(Acc* a, float g, float b);
template <>
__device__ __forceinline__ void acc_add<float>(float* a, float g, float b) { atomicAdd(a, __fmul_rn(g, b)); }
template <>
__device__ __forceinline__ void acc_add<double>(double* a, float g, float b) { atomicAdd(a, (double)g * (double)b); }

template <typename Acc>
__global__ void __launch_bounds__(256) interp_backward_kernel(int64_t npix, const float4* __restrict__ rast, int C,
                                                              const float* __restrict__ d_image,
                                                              const int* __restrict__ tri, int T, int V,
                                                              Acc* __restrict__ d_attr) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float4 r = rast[p];
    const int t = f2i(r.w) - 1;
    if (t < 0 || t >= T) return;
    const float b0 = r.x, b1 = r.y, b2 = __fsub_rn(__fsub_rn(1.f, b0), b1);
    const int v0 = __ldg(tri + 3 * t), v1 = __ldg(tri + 3 * t + 1), v2 = __ldg(tri + 3 * t + 2);
    if ((unsigned)v0 >= (unsigned)V || (unsigned)v1 >= (unsigned)V || (unsigned)v2 >= (unsigned)V) return;
    for (int d = 0; d < C; ++d) {
        const float g = d_image[p * C + d];
        acc_add<Acc>(d_attr + (int64_t)C * v0 + d, g, b0);
        acc_add<Acc>(d_attr + (int64_t)C * v1 + d, g, b1);
        acc_add<Acc>(d_attr + (int64_t)C * v2 + d, g, b2);
    }
}

// d_attr += round_to_float(acc): one rounding of each FP64 sum
__global__ void __launch_bounds__(256) finish_acc64(int64_t n, const double* __restrict__ acc, float* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __fadd_rn(out[i], __double2float_rn(acc[i]));
}

// dda.cu:258-284
__global__ void __launch_bounds__(256) dda_interp_kernel(int64_t npix, const float4* __restrict__ rast, int C,
                                                         const float* __restrict__ attr, int V,
                                                         const int2* __restrict__ edges, int E,
                                                         float* __restrict__ image) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float4 r = rast[p];
    const int e = f2i(r.w) - 1;
    if (e < 0 || e >= E) return;
    const float t1 = r.y, t0 = __fsub_rn(1.f, t1);
    const int2 ev = __ldg(edges + e);
    if ((unsigned)ev.x >= (unsigned)V || (unsigned)ev.y >= (unsigned)V) return;
    for (int d = 0; d < C; ++d)
        image[p * C + d] = __fmaf_rn(t1, __ldg(attr + (int64_t)C * ev.y + d), __fmul_rn(t0, __ldg(attr + (int64_t)C * ev.x + d)));
}

// dda.cu:300-327 (float or FP64 accumulation, as interp_backward_kernel)
template <typename Acc>
__global__ void __launch_bounds__(256) dda_interp_backward_kernel(int64_t npix, const float4* __restrict__ rast, int C,
                                                                  const float* __restrict__ d_image,
                                                                  const int2* __restrict__ edges, int E, int V,
                                                                  Acc* __restrict__ d_attr) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const float4 r = rast[p];
    const int e = f2i(r.w) - 1;
    if (e < 0 || e >= E) return;
    const float t1 = r.y, t0 = __fsub_rn(1.f, t1);
    const int2 ev = __ldg(edges + e);
    if ((unsigned)ev.x >= (unsigned)V || (unsigned)ev.y >= (unsigned)V) return;
    for (int d = 0; d < C; ++d) {
        const float g = d_image[p * C + d];
        acc_add<Acc>(d_attr + (int64_t)C * ev.x + d, g, t0);
        acc_add<Acc>(d_attr + (int64_t)C * ev.y + d, g, t1);
    }
}

// Barycentric derivatives (no counterpart in the reference, whose rasteriser outputs
// barycentrics only): d(b0, b1)/d(x, y) in pixel units at every covered pixel of rast.
// The forward's clip-space edge functions (rasterize.cu:144-156) A_i = q_j x q_k with
// q_j = (x_j - px w_j, -y_j - py w_j) are affine in (px, py):
// dA_i/dpx = w_j y_k - w_k y_j and dA_i/dpy = w_j x_k - w_k x_j for (i, j, k) cyclic, so
// db_i/dpx = (dA_i/dpx - b_i sum_m dA_m/dpx) / A, with dpx/dx = 2 / W and dpy/dy = 2 / H.
// Output (du/dx, du/dy, dv/dx, dv/dy) for (u, v) = (b0, b1); 0 where the pixel is empty.
__global__ void __launch_bounds__(256) bary_db_kernel(int B, int H, int W, Tris R, const float4* __restrict__ rast,
                                                      float4* __restrict__ db) {
    const int64_t n = (int64_t)B * H * W;
    const float sxp = __fdiv_rn(2.f, (float)W), syp = __fdiv_rn(2.f, (float)H);
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
        const float4 r = __ldg(rast + idx);
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        const int t = f2i(r.w) - 1;
        const int64_t bh = idx / W;
        const int x = (int)(idx - bh * W);
        const int b = (int)(bh / H);
        const int y = (int)(bh - (int64_t)b * H);
        if (t >= 0 && t < R.T) {
            const int i0 = __ldg(R.tri + 3 * t), i1 = __ldg(R.tri + 3 * t + 1), i2 = __ldg(R.tri + 3 * t + 2);
            if ((unsigned)i0 < (unsigned)R.V && (unsigned)i1 < (unsigned)R.V && (unsigned)i2 < (unsigned)R.V) {
                const float4* pb = R.pos4 + (int64_t)b * R.V;
                const float4 P0 = __ldg(pb + i0), P1 = __ldg(pb + i1), P2 = __ldg(pb + i2);
                const float px = __fadd_rn(-1.f, __fdiv_rn(__fmul_rn(2.f, __fadd_rn((float)x, 0.5f)), (float)W));
                const float py = __fadd_rn(-1.f, __fdiv_rn(__fmul_rn(2.f, __fadd_rn((float)y, 0.5f)), (float)H));
                const float q0x = __fmaf_rn(-px, P0.w, P0.x), q0y = __fmaf_rn(-py, P0.w, -P0.y);
                const float q1x = __fmaf_rn(-px, P1.w, P1.x), q1y = __fmaf_rn(-py, P1.w, -P1.y);
                const float q2x = __fmaf_rn(-px, P2.w, P2.x), q2y = __fmaf_rn(-py, P2.w, -P2.y);
                const float A0 = __fmaf_rn(q1x, q2y, -__fmul_rn(q1y, q2x));
                const float A1 = __fmaf_rn(q2x, q0y, -__fmul_rn(q2y, q0x));
                const float A2 = __fmaf_rn(q0x, q1y, -__fmul_rn(q0y, q1x));
                const float A = __fadd_rn(__fadd_rn(A0, A1), A2);
                if (A != 0.f) {
                    const float a0x = __fmaf_rn(P1.w, P2.y, -__fmul_rn(P2.w, P1.y));
                    const float a1x = __fmaf_rn(P2.w, P0.y, -__fmul_rn(P0.w, P2.y));
                    const float a2x = __fmaf_rn(P0.w, P1.y, -__fmul_rn(P1.w, P0.y));
                    const float a0y = __fmaf_rn(P1.w, P2.x, -__fmul_rn(P2.w, P1.x));
                    const float a1y = __fmaf_rn(P2.w, P0.x, -__fmul_rn(P0.w, P2.x));
                    const float a2y = __fmaf_rn(P0.w, P1.x, -__fmul_rn(P1.w, P0.x));
                    const float sx = __fadd_rn(__fadd_rn(a0x, a1x), a2x);
                    const float sy = __fadd_rn(__fadd_rn(a0y, a1y), a2y);
                    const float b0 = r.x, b1 = r.y;
                    o.x = __fmul_rn(__fdiv_rn(__fmaf_rn(-b0, sx, a0x), A), sxp);
                    o.y = __fmul_rn(__fdiv_rn(__fmaf_rn(-b0, sy, a0y), A), syp);
                    o.z = __fmul_rn(__fdiv_rn(__fmaf_rn(-b1, sx, a1x), A), sxp);
                    o.w = __fmul_rn(__fdiv_rn(__fmaf_rn(-b1, sy, a1y), A), syp);
                }
            }
        }
        db[idx] = o;
    }
}

}  // namespace s2c

using namespace s2c;

extern "C" s2c_status s2c_barycentric_derivatives(int B, int H, int W, int V, const float* pos, int T,
                                                  const int32_t* tri, const float* rast, float* rast_db,
                                                  s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && V >= 0 && T >= 0, "barycentric_derivatives: bad sizes");
    const int64_t n = (int64_t)B * H * W;
    if (n == 0) return S2C_OK;
    S2C_REQUIRE(rast && rast_db && (V == 0 || pos) && (T == 0 || tri), "barycentric_derivatives: null pointer");
    S2C_REQUIRE(((uintptr_t)rast & 15) == 0 && ((uintptr_t)rast_db & 15) == 0 && ((uintptr_t)pos & 15) == 0,
                "barycentric_derivatives: misaligned");
    Tris R;
    R.pos4 = (const float4*)pos;
    R.tri = tri;
    R.V = V;
    R.T = T;
    R.divT = FastDiv((uint32_t)(T > 0 ? T : 1));
    bary_db_kernel<<<grid_for(n, 256, (int64_t)num_sms() * 16), 256, 0, (cudaStream_t)stream>>>(
        B, H, W, R, (const float4*)rast, (float4*)rast_db);
    S2C_CHECK_LAUNCH("bary_db_kernel");
    return S2C_OK;
}

static Tris make_tris(int V, const float* pos, int T, const int32_t* tri) {
    Tris R;
    R.pos4 = (const float4*)pos;
    R.tri = tri;
    R.V = V;
    R.T = T;
    R.divT = FastDiv((uint32_t)(T > 0 ? T : 1));
    return R;
}

extern "C" size_t s2c_compute_triangle_rects_workspace_size(int B, int T) {
    return scan_workspace_bytes((int64_t)B * T) + 256;
}

extern "C" s2c_status s2c_compute_triangle_rects(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                                 int32_t* rects, int32_t* prefix, void* ws, size_t ws_bytes,
                                                 int64_t* num_frags, s2c_stream stream) {
    S2C_REQUIRE(H > 0 && W > 0 && B > 0 && V >= 0 && T >= 0, "compute_triangle_rects: bad sizes");
    const int64_t BT = (int64_t)B * T;
    S2C_REQUIRE(BT < (1LL << 31), "compute_triangle_rects: B*T too large");
    S2C_REQUIRE(BT == 0 || (pos && tri && rects && prefix), "compute_triangle_rects: null pointer");
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)rects & 15) == 0, "compute_triangle_rects: misaligned");
    if (!ws || ws_bytes < s2c_compute_triangle_rects_workspace_size(B, T)) {
        set_error("compute_triangle_rects: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int64_t* d_total = (int64_t*)((char*)ws + scan_workspace_bytes(BT));
    if (BT > 0) {
        tri_rects_kernel<<<grid_for(BT, 256), 256, 0, st>>>(H, W, B, make_tris(V, pos, T, tri), (int4*)rects, prefix);
        S2C_CHECK_LAUNCH("tri_rects_kernel");
    }
    if (s2c_status s = inclusive_scan_i32(prefix, BT, prefix, ws, d_total, st)) return s;
    if (s2c_status s = read_count(d_total, num_frags, st)) return s;
    if (num_frags && *num_frags > 0x7fffffffLL) {
        set_error("compute_triangle_rects: %lld bounding-box pixels exceed the int32 prefix sum", (long long)*num_frags);
        return S2C_ERR_INVALID;
    }
    return S2C_OK;
}

extern "C" s2c_status s2c_compute_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                            const int32_t* prefix, const int32_t* rects, int64_t F, int32_t* frag_pix,
                                            float* frag_attrs, s2c_stream stream) {
    S2C_REQUIRE(H > 0 && W > 0 && B > 0 && V >= 0 && T >= 0 && F >= 0, "compute_fragments: bad sizes");
    if (F == 0 || (int64_t)B * T == 0) return S2C_OK;
    S2C_REQUIRE(pos && tri && prefix && rects && frag_pix && frag_attrs, "compute_fragments: null pointer");
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)rects & 15) == 0 && ((uintptr_t)frag_attrs & 15) == 0,
                "compute_fragments: misaligned");
    tri_fragments_kernel<<<grid_for(F, 256), 256, 0, (cudaStream_t)stream>>>(
        H, W, make_tris(V, pos, T, tri), (int64_t)B * T, F, prefix, (const int4*)rects, frag_pix, (float4*)frag_attrs);
    S2C_CHECK_LAUNCH("tri_fragments_kernel");
    return S2C_OK;
}

namespace {
s2c_status list_args(const char* what, int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                     const int32_t* prefix, const int32_t* rects, int64_t F, void* ws, size_t ws_bytes, ListWs& w) {
    S2C_REQUIRE(H > 0 && W > 0 && B > 0 && V >= 0 && T >= 0 && F >= 0, "%s: bad sizes", what);
    S2C_REQUIRE(F < (1LL << 31) && (int64_t)B * T < (1LL << 31), "%s: too many bounding-box pixels", what);
    S2C_REQUIRE(F == 0 || (pos && tri && prefix && rects), "%s: null pointer", what);
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)rects & 15) == 0, "%s: misaligned", what);
    S2C_REQUIRE(ws && ((uintptr_t)ws & 15) == 0, "%s: null or misaligned workspace", what);
    const size_t need = list_carve(F, ws, ws_bytes, &w);
    S2C_REQUIRE(need <= ws_bytes, "%s: workspace of %zu bytes, need %zu", what, ws_bytes, need);
    return S2C_OK;
}
}  // namespace

extern "C" size_t s2c_count_fragments_workspace_size(int64_t num_bbox_pixels) {
    return list_carve(num_bbox_pixels < 0 ? 0 : num_bbox_pixels, nullptr, (size_t)-1, nullptr) + 256;
}

extern "C" s2c_status s2c_count_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                          const int32_t* prefix, const int32_t* rects, int64_t F, void* workspace,
                                          size_t workspace_bytes, int64_t* num_frags, s2c_stream stream) {
    ListWs w;
    if (s2c_status s = list_args("count_fragments", H, W, B, V, pos, T, tri, prefix, rects, F, workspace,
                                 workspace_bytes, w))
        return s;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nw = (F + 31) / 32;
    cudaError_t e = cudaMemsetAsync(w.mask, 0, (size_t)std::max<int64_t>(nw, 1) * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "count_fragments: memset");
    if (F > 0) {
        tri_list_kernel<false><<<list_grid(F), 256, 0, st>>>(H, W, make_tris(V, pos, T, tri), (int64_t)B * T,
                                                            (uint32_t)F, prefix, (const int4*)rects, w.mask, nullptr,
                                                            nullptr, nullptr);
        S2C_CHECK_LAUNCH("tri_list_kernel<count>");
    }
    return list_count(F, w, num_frags, st);
}

extern "C" s2c_status s2c_write_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                          const int32_t* prefix, const int32_t* rects, int64_t F, const void* workspace,
                                          size_t workspace_bytes, int32_t* frag_pix, float* frag_attrs,
                                          s2c_stream stream) {
    ListWs w;
    if (s2c_status s = list_args("write_fragments", H, W, B, V, pos, T, tri, prefix, rects, F,
                                 const_cast<void*>(workspace), workspace_bytes, w))
        return s;
    if (F == 0) return S2C_OK;
    S2C_REQUIRE(frag_pix && frag_attrs && ((uintptr_t)frag_attrs & 15) == 0, "write_fragments: bad outputs");
    cudaStream_t st = (cudaStream_t)stream;
    tri_list_kernel<true><<<list_grid(F), 256, 0, st>>>(H, W, make_tris(V, pos, T, tri), (int64_t)B * T, (uint32_t)F, prefix,
                                               (const int4*)rects, w.mask, w.wpre, frag_pix, (float4*)frag_attrs);
    S2C_CHECK_LAUNCH("tri_list_kernel<write>");
    return S2C_OK;
}

extern "C" size_t s2c_depth_test_workspace_size(int B, int H, int W) { return (size_t)B * H * W * 8 + 256; }

extern "C" s2c_status s2c_depth_test(int B, int H, int W, int64_t F, const int32_t* frag_pix, const float* frag_attrs,
                                     float* rast_out, void* ws, size_t ws_bytes, s2c_stream stream) {
    S2C_REQUIRE(B > 0 && H > 0 && W > 0 && F >= 0, "depth_test: bad sizes");
    S2C_REQUIRE(F < (1LL << 31), "depth_test: too many fragments");
    S2C_REQUIRE(rast_out && ((uintptr_t)rast_out & 15) == 0, "depth_test: rast_out must be 16-byte aligned");
    S2C_REQUIRE(F == 0 || (frag_pix && frag_attrs && ((uintptr_t)frag_attrs & 15) == 0), "depth_test: bad fragments");
    if (!ws || ws_bytes < s2c_depth_test_workspace_size(B, H, W)) {
        set_error("depth_test: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t npix = (int64_t)B * H * W;
    unsigned long long* keys = (unsigned long long*)ws;
    fill_keys<<<grid_for(npix, 256), 256, 0, st>>>(keys, npix);
    if (F > 0)
        depth_keys_kernel<<<grid_for(F, 256), 256, 0, st>>>(F, frag_pix, (const float4*)frag_attrs, B, H, W, keys);
    depth_gather_kernel<<<grid_for(npix, 256), 256, 0, st>>>(npix, keys, (const float4*)frag_attrs, F, (float4*)rast_out);
    S2C_CHECK_LAUNCH("depth_test");
    return S2C_OK;
}

extern "C" s2c_status s2c_interpolate_triangle_attributes(int B, int H, int W, int C, const float* rast, int V,
                                                          const float* attr, int T, const int32_t* tri, float* image,
                                                          s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && C >= 0 && V >= 0 && T >= 0, "interpolate_triangle_attributes: bad sizes");
    const int64_t npix = (int64_t)B * H * W;
    if (npix == 0 || C == 0) return S2C_OK;
    S2C_REQUIRE(rast && attr && tri && image && ((uintptr_t)rast & 15) == 0, "interpolate_triangle_attributes: bad pointer");
    interp_kernel<<<grid_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(npix, (const float4*)rast, C, attr, V, tri, T,
                                                                         image);
    S2C_CHECK_LAUNCH("interp_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_backward_interpolate_triangle_attributes(int B, int H, int W, int C, const float* rast,
                                                                   const float* d_image, int T, const int32_t* tri,
                                                                   int V, float* d_attr, double* acc64,
                                                                   s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && C >= 0 && V >= 0 && T >= 0,
                "backward_interpolate_triangle_attributes: bad sizes");
    const int64_t npix = (int64_t)B * H * W;
    if (npix == 0 || C == 0) return S2C_OK;
    S2C_REQUIRE(rast && d_image && tri && d_attr && ((uintptr_t)rast & 15) == 0,
                "backward_interpolate_triangle_attributes: bad pointer");
    S2C_REQUIRE(((uintptr_t)acc64 & 7) == 0, "backward_interpolate_triangle_attributes: misaligned accumulator");
    cudaStream_t st = (cudaStream_t)stream;
    if (!acc64) {
        interp_backward_kernel<float><<<grid_for(npix, 256), 256, 0, st>>>(npix, (const float4*)rast, C, d_image, tri, T,
                                                                            V, d_attr);
        S2C_CHECK_LAUNCH("interp_backward_kernel");
        return S2C_OK;
    }
    const int64_t n = (int64_t)V * C;
    if (cudaError_t e = cudaMemsetAsync(acc64, 0, (size_t)n * sizeof(double), st))
        return cuda_status(e, "backward_interpolate_triangle_attributes: clearing the accumulator");
    interp_backward_kernel<double><<<grid_for(npix, 256), 256, 0, st>>>(npix, (const float4*)rast, C, d_image, tri, T, V,
                                                                         acc64);
    S2C_CHECK_LAUNCH("interp_backward_kernel");
    finish_acc64<<<grid_for(n, 256, (int64_t)num_sms() * 8), 256, 0, st>>>(n, acc64, d_attr);
    S2C_CHECK_LAUNCH("finish_acc64");
    return S2C_OK;
}

extern "C" s2c_status s2c_dda_interpolate_attributes(int B, int H, int W, int C, const float* rast, int V,
                                                     const float* attr, int E, const int32_t* edges, float* image,
                                                     s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && C >= 0 && V >= 0 && E >= 0, "dda_interpolate_attributes: bad sizes");
    const int64_t npix = (int64_t)B * H * W;
    if (npix == 0 || C == 0) return S2C_OK;
    S2C_REQUIRE(rast && attr && edges && image && ((uintptr_t)rast & 15) == 0 && ((uintptr_t)edges & 7) == 0,
                "dda_interpolate_attributes: bad pointer");
    dda_interp_kernel<<<grid_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(npix, (const float4*)rast, C, attr, V,
                                                                             (const int2*)edges, E, image);
    S2C_CHECK_LAUNCH("dda_interp_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_backward_dda_interpolate_attributes(int B, int H, int W, int C, const float* rast,
                                                              const float* d_image, int E, const int32_t* edges, int V,
                                                              float* d_attr, double* acc64, s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && C >= 0 && V >= 0 && E >= 0,
                "backward_dda_interpolate_attributes: bad sizes");
    const int64_t npix = (int64_t)B * H * W;
    if (npix == 0 || C == 0) return S2C_OK;
    S2C_REQUIRE(rast && d_image && edges && d_attr && ((uintptr_t)rast & 15) == 0 && ((uintptr_t)edges & 7) == 0,
                "backward_dda_interpolate_attributes: bad pointer");
    S2C_REQUIRE(((uintptr_t)acc64 & 7) == 0, "backward_dda_interpolate_attributes: misaligned accumulator");
    cudaStream_t st = (cudaStream_t)stream;
    if (!acc64) {
        dda_interp_backward_kernel<float><<<grid_for(npix, 256), 256, 0, st>>>(
            npix, (const float4*)rast, C, d_image, (const int2*)edges, E, V, d_attr);
        S2C_CHECK_LAUNCH("dda_interp_backward_kernel");
        return S2C_OK;
    }
    const int64_t n = (int64_t)V * C;
    if (cudaError_t e = cudaMemsetAsync(acc64, 0, (size_t)n * sizeof(double), st))
        return cuda_status(e, "backward_dda_interpolate_attributes: clearing the accumulator");
    dda_interp_backward_kernel<double><<<grid_for(npix, 256), 256, 0, st>>>(
        npix, (const float4*)rast, C, d_image, (const int2*)edges, E, V, acc64);
    S2C_CHECK_LAUNCH("dda_interp_backward_kernel");
    finish_acc64<<<grid_for(n, 256, (int64_t)num_sms() * 8), 256, 0, st>>>(n, acc64, d_attr);
    S2C_CHECK_LAUNCH("finish_acc64");
    return S2C_OK;
}

namespace {
struct RasterWs {
    unsigned long long* keys;
    int4* rects;
    int32_t* areas;
    int32_t* prefix;
    int64_t* total;
    void* scan;
};

size_t raster_carve(int B, int H, int W, int T, bool with_keys, void* base, size_t cap, RasterWs* w) {
    Carver cv(base, cap);
    RasterWs r;
    const int64_t BT = std::max<int64_t>((int64_t)B * T, 1);
    r.keys = with_keys ? cv.take<unsigned long long>((size_t)B * H * W) : nullptr;
    r.rects = cv.take<int4>(BT);
    r.areas = cv.take<int32_t>(BT);
    r.prefix = cv.take<int32_t>(BT);
    r.total = cv.take<int64_t>(1);
    r.scan = cv.take<char>(scan_workspace_bytes(BT));
    if (w) *w = r;
    return cv.off;
}
}  // namespace

extern "C" size_t s2c_rasterize_fused_workspace_size(int B, int H, int W, int T) {
    if (B <= 0 || H <= 0 || W <= 0 || T < 0) return 256;
    return raster_carve(B, H, W, T, true, nullptr, (size_t)-1, nullptr) + 256;
}

static s2c_status rasterize_fused_impl(int B, int H, int W, int V, const float* pos, int T, const int32_t* tri,
                                       const int32_t* tri2cluster, int num_tri2cluster, int S, int32_t* bitset,
                                       uint32_t* planes, float* rast, void* workspace, size_t workspace_bytes,
                                       s2c_stream stream, bool clear_planes, int32_t* cluster_rects);

extern "C" s2c_status s2c_rasterize_fused(int B, int H, int W, int V, const float* pos, int T, const int32_t* tri,
                                          const int32_t* tri2cluster, int num_tri2cluster, int S, int32_t* bitset,
                                          float* rast, void* workspace, size_t workspace_bytes, s2c_stream stream) {
    return rasterize_fused_impl(B, H, W, V, pos, T, tri, tri2cluster, num_tri2cluster, S, bitset, nullptr, rast,
                                workspace, workspace_bytes, stream, true, nullptr);
}

extern "C" s2c_status s2c_rasterize_fused_planes(int B, int H, int W, int V, const float* pos, int T,
                                                 const int32_t* tri, const int32_t* tri2cluster, int num_tri2cluster,
                                                 int S, uint32_t* planes, float* rast, void* workspace,
                                                 size_t workspace_bytes, s2c_stream stream) {
    return rasterize_fused_impl(B, H, W, V, pos, T, tri, tri2cluster, num_tri2cluster, S, nullptr, planes, rast,
                                workspace, workspace_bytes, stream, true, nullptr);
}

extern "C" s2c_status s2c_rasterize_fused_planes_onto(int B, int H, int W, int V, const float* pos, int T,
                                                      const int32_t* tri, const int32_t* tri2cluster,
                                                      int num_tri2cluster, int S, uint32_t* planes,
                                                      int32_t* cluster_rects, void* workspace,
                                                      size_t workspace_bytes, s2c_stream stream) {
    S2C_REQUIRE(planes && cluster_rects, "rasterize_fused_planes_onto: null planes / cluster_rects");
    S2C_REQUIRE(((uintptr_t)cluster_rects & 15) == 0, "rasterize_fused_planes_onto: misaligned cluster_rects");
    return rasterize_fused_impl(B, H, W, V, pos, T, tri, tri2cluster, num_tri2cluster, S, nullptr, planes, nullptr,
                                workspace, workspace_bytes, stream, false, cluster_rects);
}

static s2c_status rasterize_fused_impl(int B, int H, int W, int V, const float* pos, int T, const int32_t* tri,
                                       const int32_t* tri2cluster, int num_tri2cluster, int S, int32_t* bitset,
                                       uint32_t* planes, float* rast, void* workspace, size_t workspace_bytes,
                                       s2c_stream stream, bool clear_planes, int32_t* cluster_rects) {
    S2C_REQUIRE(B > 0 && H > 0 && W > 0 && H <= 32768 && W <= 32768 && V >= 0 && T >= 0,
                "rasterize_fused: bad sizes");
    S2C_REQUIRE((int64_t)B * T < (1LL << 31), "rasterize_fused: B*T too large");
    S2C_REQUIRE((!bitset && !planes) || (S > 0 && (tri2cluster || num_tri2cluster == 0)),
                "rasterize_fused: bitset needs S and tri2cluster");
    S2C_REQUIRE(pos && (T == 0 || tri), "rasterize_fused: null input");
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && (!rast || ((uintptr_t)rast & 15) == 0), "rasterize_fused: misaligned");
    const int64_t npix = (int64_t)B * H * W;
    cudaStream_t st = (cudaStream_t)stream;
    RasterWs ws;
    const size_t need = raster_carve(B, H, W, T, rast != nullptr, workspace, workspace_bytes, &ws);
    S2C_REQUIRE(workspace && need <= workspace_bytes, "rasterize_fused: workspace of %zu bytes, need %zu",
                workspace_bytes, need);
    if (rast) {
        cudaError_t e = cudaMemsetAsync(ws.keys, 0xff, (size_t)npix * 8, st);
        if (e != cudaSuccess) return cuda_status(e, "rasterize_fused: memset keys");
    }
    if (bitset) {
        cudaError_t e = cudaMemsetAsync(bitset, 0, (size_t)npix * S * 4, st);
        if (e != cudaSuccess) return cuda_status(e, "rasterize_fused: memset bitset");
    }
    const int WQ = (W + 31) / 32;
    if (planes && clear_planes) {
        cudaError_t e = cudaMemsetAsync(planes, 0, (size_t)B * 32 * S * H * WQ * 4, st);
        if (e != cudaSuccess) return cuda_status(e, "rasterize_fused: memset planes");
    }
    ClusterRects CR;
    CR.r = (int4*)cluster_rects;
    CR.t2c = tri2cluster;
    CR.num_t2c = num_tri2cluster;
    CR.Kp = 32 * S;
    if (cluster_rects) {
        const int64_t n = (int64_t)B * 32 * S;
        cluster_rects_init_kernel<<<grid_for(n, 256, (int64_t)num_sms() * 8), 256, 0, st>>>(n, H, WQ, CR.r);
        S2C_CHECK_LAUNCH("cluster_rects_init_kernel");
    }
    Tris R;
    R.pos4 = (const float4*)pos;
    R.tri = tri;
    R.V = V;
    R.T = T;
    R.divT = FastDiv((uint32_t)(T > 0 ? T : 1));
    const int64_t BT = (int64_t)B * T;
    if (BT > 0 && (rast || bitset || planes)) {
        tri_rect_area_kernel<<<grid_for(BT, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(H, W, B, R, ws.rects,
                                                                                           ws.areas, CR);
        S2C_CHECK_LAUNCH("tri_rect_area_kernel");
        s2c_status s = inclusive_scan_i32(ws.areas, BT, ws.prefix, ws.scan, ws.total, st);
        if (s != S2C_OK) return s;
        FusedRaster F;
        F.B = B;
        F.H = H;
        F.W = W;
        F.S = S;
        F.R = R;
        F.t2c = tri2cluster;
        F.num_t2c = num_tri2cluster;
        F.bitset = bitset;
        F.planes = planes;
        F.WQ = WQ;
        F.keys = ws.keys;
        F.rects = ws.rects;
        F.prefix = (const uint32_t*)ws.prefix;
        F.total = ws.total;
        const size_t lut = W + H <= 8192 ? (size_t)(W + H) * sizeof(float) : 0;
        tri_fused_kernel<<<(unsigned)num_sms() * 8, 256, lut, st>>>(F);
        S2C_CHECK_LAUNCH("tri_fused_kernel");
    }
    if (rast) {
        tri_resolve_kernel<<<grid_for(npix, 256, (int64_t)num_sms() * 16), 256, 0, st>>>(B, H, W, R, ws.keys,
                                                                                           (float4*)rast);
        S2C_CHECK_LAUNCH("tri_resolve_kernel");
    }
    return S2C_OK;
}

extern "C" s2c_status s2c_msaa_resolve(int S, int H, int W, int C, const float* rast, int V, const float* attr, int T,
                                       const int32_t* tri, const float* weights, float* acc, float* count,
                                       float* alpha, s2c_stream stream) {
    S2C_REQUIRE(S > 0 && H >= 0 && W >= 0 && C >= 0 && C <= kMsaaMaxC && V >= 0 && T >= 0,
                "msaa_resolve: bad sizes (at most %d channels)", kMsaaMaxC);
    const int64_t npix = (int64_t)H * W;
    if (npix == 0) return S2C_OK;
    S2C_REQUIRE(rast && weights && count && alpha && (C == 0 || (acc && attr)) && (T == 0 || tri),
                "msaa_resolve: null pointer");
    S2C_REQUIRE(((uintptr_t)rast & 15) == 0, "msaa_resolve: misaligned rast");
    msaa_resolve_kernel<<<grid_for(npix, 256, (int64_t)num_sms() * 16), 256, 0, (cudaStream_t)stream>>>(
        S, npix, C, (const float4*)rast, attr, V, tri, T, weights, acc, count, alpha);
    S2C_CHECK_LAUNCH("msaa_resolve_kernel");
    return S2C_OK;
}
