// DDA line rasterisation of strand segments (the reference's dda.cu / rasterize.cu:474-520).
//
// The drop-in fragment path: span -> scan -> fragments -> compaction -> cluster mask,
// entry for entry the reference's _core calls, with the same per-fragment arithmetic.
// The fused segment -> bitset path lives in dda_fused.cu.
#include <algorithm>

#include "lines.cuh"
#include "scan.cuh"
#include "list.cuh"

namespace s2c {

// ---------------------------------------------------------------------------------------
// common per-primitive setup
// ---------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------
// drop-in kernels
// ---------------------------------------------------------------------------------------

// dda.cu:9-87
__global__ void __launch_bounds__(256) dda_span_kernel(int64_t P, Lines L, int H, int W, int32_t* __restrict__ counts,
                                                       float2* __restrict__ slopes, float4* __restrict__ spans) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    Prim q;
    Span s;
    if (load_prim(p, L, q)) {
        s = dda_span(q.p0, q.p1, H, W);
    } else {
        s.sx = s.sy = s.slope = s.off0 = s.off1 = s.axis = 0.f;
        s.count = 0;
    }
    counts[p] = s.count;
    slopes[p] = make_float2(s.axis, s.slope);
    spans[p] = make_float4(s.sx, s.sy, s.off0, s.off1);
}

// dda.cu:146-225: one thread per fragment, owner primitive by binary search in the
// inclusive prefix sum; the span parameters are read back from the span arrays.
__global__ void __launch_bounds__(256) dda_fragments_kernel(int64_t P, int64_t F, const int32_t* __restrict__ prefix,
                                                            Lines L, const float2* __restrict__ slopes,
                                                            const float4* __restrict__ spans, int H, int W,
                                                            int32_t* __restrict__ frag_pix,
                                                            float4* __restrict__ frag_attrs) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= F) return;
    int64_t lo = 0, hi = P;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)(uint32_t)__ldg(prefix + mid) <= idx) lo = mid + 1;
        else hi = mid;
    }
    if (lo >= P) return;
    const int64_t base = lo ? (int64_t)(uint32_t)__ldg(prefix + lo - 1) : 0;
    const int k = (int)(idx - base);
    const float2 sl = __ldg(slopes + lo);
    const float4 sp = __ldg(spans + lo);
    Span s;
    s.axis = sl.x; s.slope = sl.y; s.sx = sp.x; s.sy = sp.y; s.off0 = sp.z; s.off1 = sp.w; s.count = 0;
    float x, y;
    dda_sample(s, k, x, y);
    const int h = f2i(floorf(y)), w = f2i(floorf(x));
    if (h < 0 || h >= H || w < 0 || w >= W) return;
    Prim q;
    if (!load_prim(lo, L, q)) return;
    const float t1 = dda_t1(q.p0, q.p1, x, y, s.axis, H, W);
    const float z = dda_z(q.p0, q.p1, t1);
    if (!z_ok(z)) return;
    frag_pix[3 * idx] = q.b;
    frag_pix[3 * idx + 1] = h;
    frag_pix[3 * idx + 2] = w;
    frag_attrs[idx] = make_float4(s.axis, t1, z, (float)(q.e + 1));
}

// The compacted fragment list (what filter_valid_fragments leaves of dda_fragments_kernel's
// list, same order and values) in two passes over the same DDA step index space (list.cuh).
template <bool kWrite>
__global__ void __launch_bounds__(256) dda_list_kernel(int64_t P, uint32_t F, const int32_t* __restrict__ prefix,
                                                       Lines L, const float2* __restrict__ slopes,
                                                       const float4* __restrict__ spans, int H, int W,
                                                       uint32_t* __restrict__ mask, const int32_t* __restrict__ wpre,
                                                       int32_t* __restrict__ frag_pix,
                                                       float4* __restrict__ frag_attrs) {
    // step k of primitive o, accepted: (b, h, w) and (axis, t1, z, e + 1)
    auto step = [&](int64_t o, int k, int& h, int& w, float& axis, float& t1, float& z, Prim& q) {
        const float2 sl = __ldg(slopes + o);
        const float4 sp = __ldg(spans + o);
        Span s;
        s.axis = sl.x;
        s.slope = sl.y;
        s.sx = sp.x;
        s.sy = sp.y;
        s.off0 = sp.z;
        s.off1 = sp.w;
        s.count = 0;
        float x, y;
        dda_sample(s, k, x, y);
        h = f2i(floorf(y));
        w = f2i(floorf(x));
        if (h < 0 || h >= H || w < 0 || w >= W) return false;
        if (!load_prim(o, L, q)) return false;
        axis = s.axis;
        t1 = dda_t1(q.p0, q.p1, x, y, s.axis, H, W);
        z = dda_z(q.p0, q.p1, t1);
        return z_ok(z);
    };
    list_pass<kWrite>(
        P, F, prefix, mask, wpre,
        [&](int64_t o, int k) {
            int h, w;
            float axis, t1, z;
            Prim q;
            return step(o, k, h, w, axis, t1, z, q);
        },
        [&](int64_t o, int k, int64_t at) {
            int h = 0, w = 0;
            float axis = 0.f, t1 = 0.f, z = 0.f;
            Prim q;
            q.b = 0;
            q.e = 0;
            step(o, k, h, w, axis, t1, z, q);   // accepted in pass 1: the same values again
            frag_pix[3 * at] = q.b;
            frag_pix[3 * at + 1] = h;
            frag_pix[3 * at + 2] = w;
            frag_attrs[at] = make_float4(axis, t1, z, (float)(q.e + 1));
        });
}

// rasterize.cu:474-498 (bounds-checked: invalid views, pixels, prims or clusters are skipped)
__global__ void __launch_bounds__(256) cluster_mask_kernel(int64_t F, const int32_t* __restrict__ frag_pix,
                                                           const float4* __restrict__ frag_attrs,
                                                           const int32_t* __restrict__ p2c, int64_t num_prims, int B,
                                                           int H, int W, int S, int32_t* __restrict__ bitset) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F) return;
    const int b = frag_pix[3 * i], y = frag_pix[3 * i + 1], x = frag_pix[3 * i + 2];
    const int prim = f2i(frag_attrs[i].w) - 1;
    if (prim < 0 || prim >= num_prims) return;
    const int c = __ldg(p2c + prim);
    if (c < 0 || c >= 32 * S || b < 0 || b >= B || y < 0 || y >= H || x < 0 || x >= W) return;
    atomicOr(bitset + (((int64_t)b * H + y) * W + x) * S + (c >> 5), (int32_t)(1u << (c & 31)));
}

}  // namespace s2c

using namespace s2c;

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
s2c_status s2c::check_lines(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V, const float* pos, int E,
                               const int32_t* edges, const char* who) {
    S2C_REQUIRE(P >= 0 && P <= 0x7fffffffLL, "%s: primitive count out of range", who);
    S2C_REQUIRE(H > 0 && W > 0 && H <= 32768 && W <= 32768, "%s: resolution must be in [1, 32768]", who);
    S2C_REQUIRE(B > 0 && V >= 0 && E >= 0, "%s: bad B/V/E", who);
    S2C_REQUIRE(P == 0 || (pos && edges), "%s: null input", who);
    S2C_REQUIRE(edge_ids || P <= (int64_t)B * E, "%s: num_prims > B*E without edge_ids", who);
    S2C_REQUIRE(P == 0 || E > 0, "%s: no edges", who);
    S2C_REQUIRE(((uintptr_t)pos & 15) == 0 && ((uintptr_t)edges & 7) == 0, "%s: misaligned pos/edges", who);
    return S2C_OK;
}

extern "C" size_t s2c_dda_compute_span_workspace_size(int64_t num_prims) {
    return scan_workspace_bytes(num_prims) + 256;
}

extern "C" s2c_status s2c_dda_compute_span(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V,
                                           const float* pos, int E, const int32_t* edges, int32_t* prefix,
                                           float* slopes, float* spans, void* ws, size_t ws_bytes,
                                           int64_t* num_frags, s2c_stream stream) {
    if (s2c_status s = check_lines(P, edge_ids, H, W, B, V, pos, E, edges, "dda_compute_span")) return s;
    S2C_REQUIRE(P == 0 || (prefix && slopes && spans), "dda_compute_span: null output");
    S2C_REQUIRE(((uintptr_t)spans & 15) == 0 && ((uintptr_t)slopes & 7) == 0, "dda_compute_span: misaligned outputs");
    if (!ws || ws_bytes < s2c_dda_compute_span_workspace_size(P)) {
        set_error("dda_compute_span: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int64_t* d_total = (int64_t*)((char*)ws + scan_workspace_bytes(P));
    if (P > 0) {
        // counts go to the prefix buffer first, then are scanned in place
        dda_span_kernel<<<grid_for(P, 256), 256, 0, st>>>(P, make_lines(edge_ids, B, V, pos, E, edges), H, W, prefix,
                                                           (float2*)slopes, (float4*)spans);
        S2C_CHECK_LAUNCH("dda_span_kernel");
    }
    if (s2c_status s = inclusive_scan_i32(prefix, P, prefix, ws, d_total, st)) return s;
    if (s2c_status s = read_count(d_total, num_frags, st)) return s;
    if (num_frags && *num_frags > 0x7fffffffLL) {
        set_error("dda_compute_span: %lld fragments exceed the int32 prefix sum", (long long)*num_frags);
        return S2C_ERR_INVALID;
    }
    return S2C_OK;
}

extern "C" s2c_status s2c_dda_compute_fragments(int64_t P, int64_t F, const int32_t* prefix, const int32_t* edge_ids,
                                                const float* slopes, const float* spans, int H, int W, int B, int V,
                                                const float* pos, int E, const int32_t* edges, int32_t* frag_pix,
                                                float* frag_attrs, s2c_stream stream) {
    if (s2c_status s = check_lines(P, edge_ids, H, W, B, V, pos, E, edges, "dda_compute_fragments")) return s;
    S2C_REQUIRE(F >= 0 && F <= 0x7fffffffLL, "dda_compute_fragments: fragment count out of range");
    if (F == 0 || P == 0) return S2C_OK;
    S2C_REQUIRE(prefix && slopes && spans && frag_pix && frag_attrs, "dda_compute_fragments: null pointer");
    S2C_REQUIRE(((uintptr_t)spans & 15) == 0 && ((uintptr_t)frag_attrs & 15) == 0 && ((uintptr_t)slopes & 7) == 0,
                "dda_compute_fragments: misaligned span/slope/attribute arrays");
    dda_fragments_kernel<<<grid_for(F, 256), 256, 0, (cudaStream_t)stream>>>(
        P, F, prefix, make_lines(edge_ids, B, V, pos, E, edges), (const float2*)slopes, (const float4*)spans, H, W,
        frag_pix, (float4*)frag_attrs);
    S2C_CHECK_LAUNCH("dda_fragments_kernel");
    return S2C_OK;
}

extern "C" size_t s2c_dda_count_fragments_workspace_size(int64_t num_steps) {
    return list_carve(num_steps < 0 ? 0 : num_steps, nullptr, (size_t)-1, nullptr) + 256;
}

static s2c_status dda_list_args(const char* who, int64_t P, int64_t F, const int32_t* prefix, const int32_t* edge_ids,
                                const float* slopes, const float* spans, int H, int W, int B, int V, const float* pos,
                                int E, const int32_t* edges, void* ws, size_t ws_bytes, ListWs& w) {
    if (s2c_status s = check_lines(P, edge_ids, H, W, B, V, pos, E, edges, who)) return s;
    S2C_REQUIRE(F >= 0 && F <= 0x7fffffffLL, "%s: fragment count out of range", who);
    S2C_REQUIRE(F == 0 || (prefix && slopes && spans), "%s: null pointer", who);
    S2C_REQUIRE(((uintptr_t)spans & 15) == 0 && ((uintptr_t)slopes & 7) == 0, "%s: misaligned span/slope arrays", who);
    S2C_REQUIRE(ws && ((uintptr_t)ws & 15) == 0, "%s: null or misaligned workspace", who);
    const size_t need = list_carve(F, ws, ws_bytes, &w);
    S2C_REQUIRE(need <= ws_bytes, "%s: workspace of %zu bytes, need %zu", who, ws_bytes, need);
    return S2C_OK;
}

extern "C" s2c_status s2c_dda_count_fragments(int64_t P, int64_t F, const int32_t* prefix, const int32_t* edge_ids,
                                              const float* slopes, const float* spans, int H, int W, int B, int V,
                                              const float* pos, int E, const int32_t* edges, void* workspace,
                                              size_t workspace_bytes, int64_t* num_frags, s2c_stream stream) {
    ListWs w;
    if (s2c_status s = dda_list_args("dda_count_fragments", P, F, prefix, edge_ids, slopes, spans, H, W, B, V, pos,
                                     E, edges, workspace, workspace_bytes, w))
        return s;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(w.mask, 0, (size_t)std::max<int64_t>((F + 31) / 32, 1) * 4, st);
    if (e != cudaSuccess) return cuda_status(e, "dda_count_fragments: memset");
    if (F > 0 && P > 0) {
        dda_list_kernel<false><<<list_grid(F), 256, 0, st>>>(P, (uint32_t)F, prefix,
                                                            make_lines(edge_ids, B, V, pos, E, edges),
                                                            (const float2*)slopes, (const float4*)spans, H, W,
                                                            w.mask, nullptr, nullptr, nullptr);
        S2C_CHECK_LAUNCH("dda_list_kernel<count>");
    }
    return list_count(P > 0 ? F : 0, w, num_frags, st);
}

extern "C" s2c_status s2c_dda_write_fragments(int64_t P, int64_t F, const int32_t* prefix, const int32_t* edge_ids,
                                              const float* slopes, const float* spans, int H, int W, int B, int V,
                                              const float* pos, int E, const int32_t* edges, const void* workspace,
                                              size_t workspace_bytes, int32_t* frag_pix, float* frag_attrs,
                                              s2c_stream stream) {
    ListWs w;
    if (s2c_status s = dda_list_args("dda_write_fragments", P, F, prefix, edge_ids, slopes, spans, H, W, B, V, pos,
                                     E, edges, const_cast<void*>(workspace), workspace_bytes, w))
        return s;
    if (F == 0 || P == 0) return S2C_OK;
    S2C_REQUIRE(frag_pix && frag_attrs && ((uintptr_t)frag_attrs & 15) == 0, "dda_write_fragments: bad outputs");
    dda_list_kernel<true><<<list_grid(F), 256, 0, (cudaStream_t)stream>>>(
        P, (uint32_t)F, prefix, make_lines(edge_ids, B, V, pos, E, edges), (const float2*)slopes,
        (const float4*)spans, H, W, w.mask, w.wpre, frag_pix, (float4*)frag_attrs);
    S2C_CHECK_LAUNCH("dda_list_kernel<write>");
    return S2C_OK;
}

extern "C" s2c_status s2c_cluster_mask_from_fragments(int64_t F, const int32_t* frag_pix, const float* frag_attrs,
                                                      const int32_t* p2c, int64_t num_prims, int B, int H, int W,
                                                      int S, int32_t* bitset, s2c_stream stream) {
    S2C_REQUIRE(F >= 0 && B > 0 && H > 0 && W > 0 && S > 0, "cluster_mask_from_fragments: bad sizes");
    if (F == 0) return S2C_OK;
    S2C_REQUIRE(frag_pix && frag_attrs && p2c && bitset, "cluster_mask_from_fragments: null pointer");
    S2C_REQUIRE(((uintptr_t)frag_attrs & 15) == 0, "cluster_mask_from_fragments: misaligned frag_attrs");
    cluster_mask_kernel<<<grid_for(F, 256), 256, 0, (cudaStream_t)stream>>>(F, frag_pix, (const float4*)frag_attrs, p2c,
                                                                            num_prims, B, H, W, S, bitset);
    S2C_CHECK_LAUNCH("cluster_mask_kernel");
    return S2C_OK;
}

