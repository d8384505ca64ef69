// Card mesh topology on the host: unique undirected edges and their adjacent triangles.
//
// Reference: mesh_utils.cpp:36-95 collects, per undirected edge, the triangles containing it
// in triangle order (std::unordered_map<EdgeKey, vector<int>>) and emits the edges in the
// map's iteration order, which is implementation-defined.  Here the half-edges are sorted
// by (min vertex, max vertex, triangle) -- a stable order any platform reproduces -- and
// each run of equal keys becomes one edge whose first two triangles are the run's first two
// entries, which is the reference's push_back order for that edge.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "s2c.h"

namespace s2c {
void set_error(const char* fmt, ...);
}

extern "C" S2C_API s2c_status s2c_build_edges_from_triangles(int T, const int32_t* tri, int32_t* edges,
                                                             int32_t* edge2tri, int64_t* num_edges) {
    if (T < 0 || !num_edges || (T > 0 && (!tri || !edges || !edge2tri))) {
        s2c::set_error("build_edges_from_triangles: invalid arguments (T=%d)", T);
        return S2C_ERR_INVALID;
    }
    struct Half {
        int32_t lo, hi, t;
    };
    std::vector<Half> h((size_t)T * 3);
    for (int t = 0; t < T; ++t) {
        const int32_t* v = tri + (size_t)t * 3;
        for (int k = 0; k < 3; ++k) {
            const int32_t a = v[k], b = v[(k + 1) % 3];
            h[(size_t)t * 3 + k] = {a < b ? a : b, a < b ? b : a, t};
        }
    }
    // (lo, hi) major, triangle minor: sort by the 64-bit key with a stable sort, since the
    // half-edges were written in triangle order
    std::stable_sort(h.begin(), h.end(), [](const Half& x, const Half& y) {
        return x.lo != y.lo ? x.lo < y.lo : x.hi < y.hi;
    });
    int64_t E = 0;
    for (size_t i = 0; i < h.size();) {
        size_t j = i + 1;
        while (j < h.size() && h[j].lo == h[i].lo && h[j].hi == h[i].hi) ++j;
        edges[2 * E] = h[i].lo;
        edges[2 * E + 1] = h[i].hi;
        edge2tri[2 * E] = h[i].t;
        edge2tri[2 * E + 1] = j - i >= 2 ? h[i + 1].t : -1;
        ++E;
        i = j;
    }
    *num_edges = E;
    return S2C_OK;
}

// Vertex adjacency (CSR) of an undirected edge list, as the uniform Laplacian of
// optimizer.py:70-99 sees it: neighbour pairs are unique (torch.unique over the pairs), a
// self-loop (v, v) makes v its own neighbour once (it adds to the degree and cancels in
// L p).  Neighbours of v are listed in the order of their first edge.  offsets has
// num_verts + 1 entries, adj at most 2 * E; *num_adj receives the count written.
extern "C" S2C_API s2c_status s2c_build_vertex_adjacency(int num_verts, int E, const int32_t* edges,
                                                        int32_t* offsets, int32_t* adj, int64_t* num_adj) {
    if (num_verts < 0 || E < 0 || !offsets || !num_adj || (E > 0 && (!edges || !adj))) {
        s2c::set_error("build_vertex_adjacency: invalid arguments (V=%d, E=%d)", num_verts, E);
        return S2C_ERR_INVALID;
    }
    std::vector<std::vector<int32_t>> nb((size_t)num_verts);
    auto add = [&](int32_t a, int32_t b) {
        for (int32_t u : nb[a])
            if (u == b) return;
        nb[a].push_back(b);
    };
    for (int e = 0; e < E; ++e) {
        const int32_t a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || a >= num_verts || b < 0 || b >= num_verts) {
            s2c::set_error("build_vertex_adjacency: edge %d = (%d, %d) outside [0, %d)", e, a, b, num_verts);
            return S2C_ERR_INVALID;
        }
        add(a, b);
        if (b != a) add(b, a);
    }
    int64_t n = 0;
    offsets[0] = 0;
    for (int v = 0; v < num_verts; ++v) {
        for (int32_t u : nb[v]) adj[n++] = u;
        offsets[v + 1] = (int32_t)n;
    }
    *num_adj = n;
    return S2C_OK;
}
