// Test infrastructure: a C entry point over the reference's own host edge builder
// (mesh_utils.cpp:36-95, compiled unmodified beside this file by build_ref.sh) so the
// CPU tests can compare libs2c's builder with it.  Returns the number of edges written
// (rows of edges / edge2tri, in the reference's hash-map order), or -1 if cap is too small.
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "hair_loader.h"

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

// The reference's own loaders (hair_loader.cpp) and serialisation: counts first
// (points == nullptr), then the arrays.
extern "C" int64_t ref_load_strands(const char* path, int kind, int32_t* counts, float* points, int64_t* num_points) {
    strns2cards::StrandsPoints sp = kind == 0 ? strns2cards::load_bin(path)
                                   : kind == 1 ? strns2cards::load_usc_data(path)
                                               : strns2cards::load_hair(path);
    size_t ns = 0, np = 0;
    int* c = nullptr;
    float* p = nullptr;
    strns2cards::serialize_strands(sp, ns, c, np, p);
    *num_points = (int64_t)np;
    if (counts && points) {
        std::memcpy(counts, c, 4 * ns);
        std::memcpy(points, p, 12 * np);
    }
    delete[] c;
    delete[] p;
    return (int64_t)ns;
}

extern "C" void ref_resample(int ns, const int32_t* counts, const float* points, int target, float* out) {
    strns2cards::resample_strands_by_arclength(ns, counts, points, target, out);
}
