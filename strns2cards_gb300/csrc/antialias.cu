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

#include "common.cuh"

namespace s2c {

struct Mesh {
    const float4* __restrict__ pos4;  // (B, V)
    const int* __restrict__ tri;      // (T, 3)
    const int2* __restrict__ edges;   // (E)
    const int2* __restrict__ e2t;     // (E)
    int V, T, E;
    FastDiv divE;
};

__device__ __forceinline__ int third_vertex(const int* __restrict__ tri, int t, int v0, int v1) {
    const int i0 = __ldg(tri + 3 * t), i1 = __ldg(tri + 3 * t + 1), i2 = __ldg(tri + 3 * t + 2);
    return (i0 != v0 && i0 != v1) ? i0 : (i1 != v0 && i1 != v1) ? i1 : (i2 != v0 && i2 != v1) ? i2 : -1;
}

// antialias.cu:29-35 without the final multiply: (1 + x/w, 1 - y/w)
__device__ __forceinline__ float2 ndc_a(float4 p) {
    return make_float2(__fadd_rn(1.f, __fdiv_rn(p.x, p.w)), __fsub_rn(1.f, __fdiv_rn(p.y, p.w)));
}

// antialias.cu:38-94
__global__ void __launch_bounds__(256) mark_edges_kernel(int H, int W, int B, Mesh M, int32_t* __restrict__ prim_ids,
                                                         float2* __restrict__ normals) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * M.E) return;
    const int b = (int)M.divE.div((uint32_t)idx);
    const int e = (int)idx - b * M.E;
    const int2 ev = __ldg(M.edges + e);
    if ((unsigned)ev.x >= (unsigned)M.V || (unsigned)ev.y >= (unsigned)M.V) return;
    const float4* pb = M.pos4 + (int64_t)b * M.V;
    const float hh = __fmul_rn((float)H, 0.5f), hw = __fmul_rn((float)W, 0.5f);
    const float2 a0 = ndc_a(__ldg(pb + ev.x)), a1 = ndc_a(__ldg(pb + ev.y));
    const float x0 = __fmul_rn(hw, a0.x), y0 = __fmul_rn(hh, a0.y);
    const float dx = __fmaf_rn(hw, a1.x, -x0), dy = __fmaf_rn(hh, a1.y, -y0);
    const float len = __fsqrt_rn(__fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
    if (len == 0.f) return;
    const float nx = __fdiv_rn(-dy, len), ny = __fdiv_rn(dx, len);
    float d[2] = {0.f, 0.f};
    const int2 tt = __ldg(M.e2t + e);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int t = i ? tt.y : tt.x;
        if (t < 0 || t >= M.T) continue;
        const int v2 = third_vertex(M.tri, t, ev.x, ev.y);
        if ((unsigned)v2 >= (unsigned)M.V) continue;  // degenerate triangle (the reference reads out of bounds)
        const float2 a2 = ndc_a(__ldg(pb + v2));
        d[i] = __fmaf_rn(nx, __fmaf_rn(hw, a2.x, -x0), __fmul_rn(ny, __fmaf_rn(hh, a2.y, -y0)));
    }
    if (__fmul_rn(d[0], d[1]) >= 0.f) prim_ids[idx] = (int32_t)idx;
    const float sign = __fmul_rn(2.f, __fsub_rn(0.5f, (float)(d[0] > 0.f || d[1] > 0.f)));
    normals[idx] = make_float2(__fmul_rn(sign, nx), __fmul_rn(sign, ny));
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
    float kr, rho;
};

__device__ __forceinline__ int bit_of(const int32_t* __restrict__ bits, int64_t pix, int S, int c) {
    return (__ldg(bits + pix * S + (c >> 5)) >> (c & 31)) & 1;
}

// antialias.cu:121-279, one warp per fragment
__global__ void __launch_bounds__(256) aa_backward_kernel(AAArgs A) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float fH = (float)A.H, fW = (float)A.W;
    for (int64_t i = warp0; i < A.F; i += nwarps) {
        // every lane evaluates the (uniform) fragment set-up
        const int b = A.frag_pix[3 * i], h = A.frag_pix[3 * i + 1], w = A.frag_pix[3 * i + 2];
        const float4 fa = A.frag_attrs[i];
        const int e = f2i(fa.w) - 1;
        if (e < 0 || e >= A.E || b < 0 || b >= A.B || h < 0 || h >= A.H || w < 0 || w >= A.W) continue;
        const float t1 = fa.y, t0 = __fsub_rn(1.f, t1);
        const int2 ev = __ldg(A.edges + e);
        if ((unsigned)ev.x >= (unsigned)A.V || (unsigned)ev.y >= (unsigned)A.V) continue;
        const float4 p0 = __ldg(A.pos4 + (int64_t)b * A.V + ev.x), p1 = __ldg(A.pos4 + (int64_t)b * A.V + ev.y);
        const float px = __fmaf_rn(t0, p0.x, __fmul_rn(t1, p1.x));
        const float py = __fmaf_rn(t0, p0.y, __fmul_rn(t1, p1.y));
        const float pw = __fmaf_rn(t0, p0.w, __fmul_rn(t1, p1.w));
        const float fx = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(1.f, __fdiv_rn(px, pw))), fW);
        const float fy = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(1.f, __fdiv_rn(py, pw))), fH);
        const float2 nrm = __ldg(A.normals + (int64_t)b * A.E + e);
        const float rx = __fsub_rn(fx, floorf(fx)), ry = __fsub_rn(fy, floorf(fy));
        int nh = h, nw = w;
        float dot;
        if (fa.x == 0.f) {
            if (!isfinite(rx) || fabsf(__fsub_rn(rx, 0.5f)) >= 1e-4f) continue;
            const int d = 2 * (int)(ry > 0.5f) - 1;
            nh += d;
            dot = __fmul_rn((float)d, nrm.y);
        } else {
            if (!isfinite(ry) || fabsf(__fsub_rn(ry, 0.5f)) >= 1e-4f) continue;
            const int d = 2 * (int)(rx > 0.5f) - 1;
            nw += d;
            dot = __fmul_rn((float)d, nrm.x);
        }
        if (nw < 0 || nw >= A.W || nh < 0 || nh >= A.H || dot == 0.f) continue;
        const int c = __ldg(A.e2c + e);
        if (c < 0 || c >= 32 * A.S) continue;
        const int64_t img = (int64_t)b * A.H * A.W;
        const int c01 = 1 - (dot > 0.f ? bit_of(A.bitset, img + (int64_t)nh * A.W + nw, A.S, c)
                                       : bit_of(A.bitset, img + (int64_t)h * A.W + w, A.S, c));
        if (c01 == 0) continue;
        // Gaussian window (antialias.cu:121-176), taps spread over the warp
        const int R = f2i(floorf(A.kr));
        const int cw = f2i(floorf(fx)), ch = f2i(floorf(fy));
        const int h0 = max(ch - R, 0), h1 = min(ch + R, A.H - 1) + 1;
        const int w0 = max(cw - R, 0), w1 = min(cw + R, A.W - 1) + 1;
        const int ww = w1 - w0, taps = ww > 0 && h1 > h0 ? ww * (h1 - h0) : 0;
        const float sigma = __fdiv_rn(A.kr, 4.f);
        const float cc = __fdiv_rn(1.f, __fmul_rn(__fmul_rn(__fmul_rn(sigma, sigma), 2.f), 3.14159265358979323846f));
        const float alpha = __fdiv_rn(0.5f, __fmul_rn(sigma, sigma));
        const float kr2 = __fmul_rn(A.kr, A.kr);
        double acc = 0.0;
        for (int j = lane; j < taps; j += 32) {
            const int th = h0 + j / ww, tw = w0 + j % ww;
            const int64_t pix = img + (int64_t)th * A.W + tw;
            const int c0 = bit_of(A.bitset, pix, A.S, c), c1 = bit_of(A.target, pix, A.S, c);
            if (c0 == c1) continue;
            const float dx = __fsub_rn(__fadd_rn((float)tw, 0.5f), fx);
            const float dy = __fsub_rn(__fadd_rn((float)th, 0.5f), fy);
            const float n2 = __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
            if (!(n2 < kr2)) continue;
            const double wgt = (double)cc * (double)expf(-alpha * n2);
            acc += wgt * (double)(c0 - c1) * (c1 == 0 ? (double)A.rho : 1.0);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane != 0) continue;
        const double dc = (double)c01 * acc;
        if (dc == 0.0) continue;
        if (A.acc64) {
            // chain rule and accumulation in FP64 (no cancellation loss across fragments)
            const double dxd = dc * 0.5 * (double)fW * (double)nrm.x;
            const double dyd = dc * -0.5 * (double)fH * (double)nrm.y;
            const double pwd = (double)pw;
            const double qx = dxd / pwd, qy = dyd / pwd;
            const double qw = (dxd * (double)px + dyd * (double)py) / (pwd * pwd);
            if (!isfinite(qx) || !isfinite(qy) || !isfinite(qw)) continue;
            double* a0 = A.acc64 + ((int64_t)b * A.V + ev.x) * 3;
            double* a1 = A.acc64 + ((int64_t)b * A.V + ev.y) * 3;
            atomicAdd(a0 + 0, qx * (double)t0);
            atomicAdd(a0 + 1, qy * (double)t0);
            atomicAdd(a0 + 2, qw * (double)t0);
            atomicAdd(a1 + 0, qx * (double)t1);
            atomicAdd(a1 + 1, qy * (double)t1);
            atomicAdd(a1 + 2, qw * (double)t1);
            continue;
        }
        const float dcf = (float)dc;
        const float dx = __fmul_rn(__fmul_rn(__fmul_rn(dcf, 0.5f), fW), nrm.x);
        const float dy = __fmul_rn(__fmul_rn(__fmul_rn(dcf, -0.5f), fH), nrm.y);
        const float dpx = __fdiv_rn(dx, pw), dpy = __fdiv_rn(dy, pw);
        const float dpw = __fdiv_rn(__fmaf_rn(dx, px, __fmul_rn(dy, py)), __fmul_rn(pw, pw));
        if (!isfinite(dpx) || !isfinite(dpy) || !isfinite(dpw)) continue;
        float* g0 = A.d_pos + ((int64_t)b * A.V + ev.x) * 4;
        float* g1 = A.d_pos + ((int64_t)b * A.V + ev.y) * 4;
        atomicAdd(g0 + 0, __fmul_rn(dpx, t0));
        atomicAdd(g0 + 1, __fmul_rn(dpy, t0));
        atomicAdd(g0 + 3, __fmul_rn(dpw, t0));
        atomicAdd(g1 + 0, __fmul_rn(dpx, t1));
        atomicAdd(g1 + 1, __fmul_rn(dpy, t1));
        atomicAdd(g1 + 3, __fmul_rn(dpw, t1));
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
