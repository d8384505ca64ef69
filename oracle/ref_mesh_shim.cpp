// Test infrastructure: a C entry point over the reference's own host edge builder
// (mesh_utils.cpp:36-95, compiled unmodified beside this file by build_ref.sh) so the
// CPU tests can compare libs2c's builder with it.  Returns the number of edges written
// (rows of edges / edge2tri, in the reference's hash-map order), or -1 if cap is too small.
#include <cstdint>
#include <vector>

namespace strns2cards {
void build_edges_from_triangles(int T, const int* tri, std::vector<int>& edges_out,
                                std::vector<int>& edge2tri_out);
}

extern "C" int64_t ref_build_edges_from_triangles(int T, const int32_t* tri, int32_t* edges,
                                                  int32_t* edge2tri, int64_t cap) {
    std::vector<int> e, t;
    strns2cards::build_edges_from_triangles(T, tri, e, t);
    const int64_t n = (int64_t)e.size() / 2;
    if (n > cap) return -1;
    for (int64_t i = 0; i < 2 * n; ++i) {
        edges[i] = e[i];
        edge2tri[i] = t[i];
    }
    return n;
}
