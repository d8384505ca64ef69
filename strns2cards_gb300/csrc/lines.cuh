// Segment inputs shared by the DDA kernels (dda.cu, dda_fused.cu).
#pragma once
#include "common.cuh"

namespace s2c {

struct Prim {
    int b, e;
    float4 p0, p1;
};

// Segment inputs shared by every DDA kernel
struct Lines {
    const int32_t* __restrict__ edge_ids;  // nullptr: primitive p is edge id p
    const float4* __restrict__ pos4;       // (B, V) homogeneous positions
    const int2* __restrict__ edges2;       // (E) vertex pairs
    int E, V;
    int64_t BE;                            // B * E
    FastDiv divE;
};

// Loads primitive p.  Ids outside [0, B*E) and vertex indices outside [0, V) (which the
// reference would read out of bounds) make the primitive empty.
__device__ __forceinline__ bool load_prim(int64_t p, const Lines& L, Prim& q) {
    const int64_t eid = L.edge_ids ? (int64_t)__ldg(L.edge_ids + p) : p;
    if (eid < 0 || eid >= L.BE) return false;
    // eid < 2^31 here (edge ids are int32 and primitive counts are capped at 2^31 - 1)
    q.b = L.BE == L.E ? 0 : (int)L.divE.div((uint32_t)eid);
    q.e = (int)eid - q.b * L.E;
    const int2 ev = __ldg(L.edges2 + q.e);
    if ((unsigned)ev.x >= (unsigned)L.V || (unsigned)ev.y >= (unsigned)L.V) return false;
    const int64_t vb = (int64_t)q.b * L.V;
    q.p0 = __ldg(L.pos4 + vb + ev.x);
    q.p1 = __ldg(L.pos4 + vb + ev.y);
    return true;
}

inline Lines make_lines(const int32_t* edge_ids, int B, int V, const float* pos, int E, const int32_t* edges) {
    Lines L;
    L.edge_ids = edge_ids;
    L.pos4 = (const float4*)pos;
    L.edges2 = (const int2*)edges;
    L.E = E;
    L.V = V;
    L.BE = (int64_t)B * E;
    L.divE = FastDiv((uint32_t)(E > 0 ? E : 1));
    return L;
}

// host-side argument checks shared by the DDA entry points
s2c_status check_lines(int64_t P, const int32_t* edge_ids, int H, int W, int B, int V, const float* pos, int E,
                       const int32_t* edges, const char* who);

}  // namespace s2c
