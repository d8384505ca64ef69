// Card mesh edges on the device: the unique undirected edges of a triangle list and, per
// edge, its first two triangles (the reference's build_edges_from_triangles,
// mesh_utils.cpp:36-95, on the host with an unordered_map whose iteration order is
// implementation-defined).
//
// The order is the host builder's (mesh.cpp): edges by (min vertex, max vertex), each edge's
// triangles in triangle order -- the reference's push_back order for that edge.  Steps, all
// on the stream, deterministic:
//   1. count the half-edges (3 per triangle) per min vertex;
//   2. scan the counts into buckets and scatter each half-edge into its min vertex's bucket;
//   3. order every bucket by (max vertex, half-edge index): one warp per bucket counts, for
//      each entry, the entries with a smaller key (keys are unique, so the counts are a
//      permutation);
//   4. flag the first half-edge of every (min, max) run, scan the flags, and write each run
//      as one edge with the triangles of its first two half-edges.
// Half-edges with a vertex outside [0, num_verts) are left out and counted.
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"

namespace s2c {
namespace {

struct HalfEdge {
    int32_t lo, hi;
};

__device__ __forceinline__ HalfEdge half_edge(const int32_t* __restrict__ tri, int64_t h) {
    const int64_t t = h / 3;
    const int k = (int)(h - 3 * t);
    const int32_t a = tri[3 * t + k], b = tri[3 * t + (k == 2 ? 0 : k + 1)];
    return HalfEdge{a < b ? a : b, a < b ? b : a};
}

__device__ __forceinline__ bool in_range(HalfEdge e, int V) { return e.lo >= 0 && e.hi < V; }

__global__ void edge_count_kernel(int64_t H, const int32_t* __restrict__ tri, int V, int32_t* __restrict__ cnt,
                                  int32_t* __restrict__ bad) {
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < H; h += (int64_t)gridDim.x * blockDim.x) {
        const HalfEdge e = half_edge(tri, h);
        if (in_range(e, V)) atomicAdd(cnt + e.lo, 1);
        else atomicAdd(bad, 1);
    }
}

__global__ void edge_scatter_kernel(int64_t H, const int32_t* __restrict__ tri, int V,
                                    const int32_t* __restrict__ cnt, const int32_t* __restrict__ incl,
                                    int32_t* __restrict__ fill, int32_t* __restrict__ bucket) {
    for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < H; h += (int64_t)gridDim.x * blockDim.x) {
        const HalfEdge e = half_edge(tri, h);
        if (!in_range(e, V)) continue;
        const int32_t pos = incl[e.lo] - cnt[e.lo] + atomicAdd(fill + e.lo, 1);
        bucket[pos] = (int32_t)h;
    }
}

// key of a bucket entry: (max vertex, half-edge index), unique
__device__ __forceinline__ uint64_t bucket_key(const int32_t* __restrict__ tri, int32_t h) {
    return ((uint64_t)(uint32_t)half_edge(tri, h).hi << 32) | (uint32_t)h;
}

__global__ void edge_rank_kernel(int V, const int32_t* __restrict__ tri, const int32_t* __restrict__ cnt,
                                 const int32_t* __restrict__ incl, const int32_t* __restrict__ bucket,
                                 int32_t* __restrict__ sorted) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < V; v += nw) {
        const int32_t d = cnt[v], b = incl[v] - d;
        for (int32_t i0 = 0; i0 < d; i0 += 32) {
            const int32_t i = i0 + lane;
            const int32_t hi_ = i < d ? bucket[b + i] : 0;
            const uint64_t ki = i < d ? bucket_key(tri, hi_) : ~0ull;
            int32_t rank = 0;
            for (int32_t j0 = 0; j0 < d; j0 += 32) {
                const uint64_t kj = j0 + lane < d ? bucket_key(tri, bucket[b + j0 + lane]) : ~0ull;
                const int m = min(32, d - j0);
                for (int k = 0; k < m; ++k) rank += __shfl_sync(0xffffffffu, kj, k) < ki ? 1 : 0;
            }
            if (i < d) sorted[b + rank] = hi_;
        }
    }
}

// flag[q] = 1 where position q starts a (min, max) run (q < n, n = valid half-edges)
__global__ void edge_flag_kernel(int64_t H, const int32_t* __restrict__ tri, const int32_t* __restrict__ sorted,
                                 const int64_t* __restrict__ d_n, int32_t* __restrict__ flag) {
    const int64_t n = *d_n;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < H; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t f = 0;
        if (q < n) {
            const HalfEdge e = half_edge(tri, sorted[q]);
            if (q == 0) {
                f = 1;
            } else {
                const HalfEdge p = half_edge(tri, sorted[q - 1]);
                f = (p.lo != e.lo || p.hi != e.hi) ? 1 : 0;
            }
        }
        flag[q] = f;
    }
}

__global__ void edge_emit_kernel(int64_t H, const int32_t* __restrict__ tri, const int32_t* __restrict__ sorted,
                                 const int64_t* __restrict__ d_n, const int32_t* __restrict__ flag,
                                 const int32_t* __restrict__ eid, int32_t* __restrict__ edges,
                                 int32_t* __restrict__ edge2tri) {
    const int64_t n = *d_n;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[q]) continue;
        const int64_t e = (int64_t)eid[q] - 1;
        const HalfEdge he = half_edge(tri, sorted[q]);
        edges[2 * e] = he.lo;
        edges[2 * e + 1] = he.hi;
        edge2tri[2 * e] = sorted[q] / 3;
        int32_t second = -1;
        if (q + 1 < n) {
            const HalfEdge nx = half_edge(tri, sorted[q + 1]);
            if (nx.lo == he.lo && nx.hi == he.hi) second = sorted[q + 1] / 3;
        }
        edge2tri[2 * e + 1] = second;
    }
}

struct EdgeWs {
    int32_t *cnt, *fill, *incl, *bucket, *sorted, *flag, *eid, *bad;
    int64_t* d_n;
    void* scan;
};

size_t edge_ws_layout(int64_t H, int V, char* base, EdgeWs* w) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += align_up(bytes, 256);
        return p;
    };
    const size_t nv = (size_t)std::max(V, 1), nh = (size_t)std::max<int64_t>(H, 1);
    EdgeWs t;
    t.cnt = (int32_t*)take(4 * nv);
    t.fill = (int32_t*)take(4 * nv);
    t.bad = (int32_t*)take(4);
    t.incl = (int32_t*)take(4 * nv);
    t.bucket = (int32_t*)take(4 * nh);
    t.sorted = (int32_t*)take(4 * nh);
    t.flag = (int32_t*)take(4 * nh);
    t.eid = (int32_t*)take(4 * nh);
    t.d_n = (int64_t*)take(8);
    t.scan = take(scan_workspace_bytes(std::max<int64_t>((int64_t)nv, (int64_t)nh)));
    if (w) *w = t;
    return off;
}

}  // namespace
}  // namespace s2c

using namespace s2c;

extern "C" S2C_API size_t s2c_build_edges_device_workspace_size(int T, int num_verts) {
    return edge_ws_layout(3 * (int64_t)std::max(T, 0), std::max(num_verts, 0), nullptr, nullptr);
}

extern "C" S2C_API s2c_status s2c_build_edges_device(int T, const int32_t* tri, int num_verts, int32_t* edges,
                                                     int32_t* edge2tri, int64_t* num_edges, int32_t* num_bad,
                                                     void* workspace, size_t workspace_bytes, s2c_stream stream) {
    S2C_REQUIRE(T >= 0 && num_verts >= 0, "build_edges_device: bad sizes (T=%d, num_verts=%d)", T, num_verts);
    S2C_REQUIRE(num_edges && num_bad, "build_edges_device: null count outputs");
    S2C_REQUIRE(3 * (int64_t)T < (int64_t)INT32_MAX, "build_edges_device: %d triangles exceed the int32 half-edge index", T);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t H = 3 * (int64_t)T;
    if (H == 0) {
        cudaMemsetAsync(num_edges, 0, sizeof(int64_t), st);
        cudaMemsetAsync(num_bad, 0, sizeof(int32_t), st);
        return cuda_status(cudaGetLastError(), "build_edges_device: memset");
    }
    S2C_REQUIRE(tri && edges && edge2tri && workspace, "build_edges_device: null pointer");
    EdgeWs w;
    const size_t need = edge_ws_layout(H, num_verts, (char*)workspace, &w);
    if (workspace_bytes < need) {
        set_error("build_edges_device: workspace of %zu bytes, need %zu", workspace_bytes, need);
        return S2C_ERR_WORKSPACE;
    }
    const int V = std::max(num_verts, 1);
    cudaMemsetAsync(w.cnt, 0, 4 * (size_t)V, st);
    cudaMemsetAsync(w.fill, 0, 4 * (size_t)V, st);
    cudaMemsetAsync(w.bad, 0, 4, st);
    const unsigned gh = grid_for(H, 256, (int64_t)num_sms() * 16);
    edge_count_kernel<<<gh, 256, 0, st>>>(H, tri, num_verts, w.cnt, w.bad);
    s2c_status rc = inclusive_scan_i32(w.cnt, V, w.incl, w.scan, w.d_n, st);
    if (rc != S2C_OK) return rc;
    edge_scatter_kernel<<<gh, 256, 0, st>>>(H, tri, num_verts, w.cnt, w.incl, w.fill, w.bucket);
    edge_rank_kernel<<<grid_for(V, 8, (int64_t)num_sms() * 16), 256, 0, st>>>(num_verts, tri, w.cnt, w.incl, w.bucket,
                                                                                w.sorted);
    edge_flag_kernel<<<gh, 256, 0, st>>>(H, tri, w.sorted, w.d_n, w.flag);
    rc = inclusive_scan_i32(w.flag, H, w.eid, w.scan, num_edges, st);
    if (rc != S2C_OK) return rc;
    edge_emit_kernel<<<gh, 256, 0, st>>>(H, tri, w.sorted, w.d_n, w.flag, w.eid, edges, edge2tri);
    cudaMemcpyAsync(num_bad, w.bad, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    S2C_CHECK_LAUNCH("build_edges_device");
    return S2C_OK;
}
