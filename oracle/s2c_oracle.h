/*
 * CPU oracle for the strands-to-cards raster path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CUDA kernels (pystrns2cards/src/ *.cu files).  It is
 * used by tests/ as the checker, by __graft_entry__.smoke() as the checker, and by
 * bench.py as the timed CPU baseline.  Nothing in the product links it.
 *
 * Integer / coverage work (fragment pixels, bitsets, silhouette decisions, triangle
 * coverage) is an FP32 bit-mirror: every float operation of the reference is restated in
 * the same order, compiled with -ffp-contract=off, and every multiply-add that nvcc may
 * contract into an FMA is written as an explicit fmaf() or left split according to the
 * "arithmetic model" flags below.  The model is pinned against the outputs of the
 * reference's own kernels (tests/golden/, produced by tests/golden/make_golden.py).
 *
 * Float outputs that the reference computes with approximate intrinsics or atomics
 * (antialias gradient, interpolation, smoothing, skinning) are evaluated in FP64 from the
 * same formulas, with the FP32-mirrored decisions (cutoffs, eps tests).
 */
#ifndef S2C_ORACLE_H
#define S2C_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic-model flags: which reference multiply-adds are treated as fused.  The default
 * (all of SPAN, PERSP, TRI_RECT, TRI_Q, TRI_A, AA) reproduces every integer output and
 * every FP32 span/slope/t1/z/barycentric/normal value of the reference kernels bit for
 * bit on the golden vectors.  Two-term and three-term dot products have fixed shapes:
 *   dda.cu:212-213         t0*a + t1*b              -> fma(t1, b, t0*a)
 *   rasterize.cu:158       A0 z0 + A1 z1 + A2 z2    -> fma(A2, z2, fma(A1, z1, A0*z0))
 *   rasterize.cu:159       A0 w0 + A1 w1 + A2 w2    -> fma(A2, w2, fma(A0, w0, A1*w1))
 *   antialias.cu:60-62     x1 - x0 (x = W/2 (1+ndc)) -> fma(W/2, 1 + ndc_x1, -x0)
 * (set_zvariant() switches the shapes; it exists only to re-run the pinning sweep). */
#define OR_FMA_DDA_SPAN     (1 << 0)  /* dda.cu:57,77   start_minor = fma(slope, start_major - p0_major, p0_minor) */
#define OR_FMA_DDA_STEP     (1 << 1)  /* dda.cu:190-193 minor = fma(d, slope, start_minor)                         */
#define OR_FMA_DDA_PERSP    (1 << 2)  /* dda.cu:130-137 p_major - q*w as fma(-q, w, p_major)                        */
#define OR_FMA_TRI_RECT     (1 << 4)  /* rasterize.cu:37-38 1 +/- p*inv_w as fma                                    */
#define OR_FMA_TRI_Q        (1 << 5)  /* rasterize.cu:144-146 q = p - pc*w as fma(-pc, w, p)                         */
#define OR_FMA_TRI_A        (1 << 6)  /* rasterize.cu:148-150 a*b - c*d as fma(a, b, -(c*d))                          */
#define OR_FMA_TRI_A_ALT    (1 << 7)  /* ... as fma(-c, d, a*b) instead (when OR_FMA_TRI_A is clear)                  */
#define OR_FMA_AA           (1 << 9)  /* antialias.cu: lengths, dots, interpolation, window norms as fma             */

int  or_version(void);
void or_set_model(int flags);
int  or_get_model(void);
void or_set_threads(int n);
void or_set_zvariant(int dda, int tri_z, int tri_w);
void or_set_aavariant(int v);

/* ---- DDA line raster (dda.cu) ---------------------------------------------------- */
void or_dda_span(int64_t P, const int32_t* edge_ids, int H, int W, int V, const float* pos,
                 int E, const int32_t* edges, int32_t* counts, float* slopes, float* spans);
/* per-prim restatement of dda_compute_fragments_kernel; prefix = inclusive int32 scan */
void or_dda_fragments(int64_t P, const int32_t* prefix, const int32_t* edge_ids,
                      const float* slopes, const float* spans, int H, int W, int V,
                      const float* pos, int E, const int32_t* edges,
                      int32_t* frag_pix, float* frag_attrs);
/* fused DDA -> cluster bitset (bitset is zeroed here); edge_ids may be NULL = all B*E */
void or_dda_cluster_bitset(int B, int H, int W, int V, const float* pos, int E,
                           const int32_t* edges, const int32_t* edge_ids, int64_t P,
                           const int32_t* prim2cluster, int S, int32_t* bitset);

/* ---- triangles (rasterize.cu) ---------------------------------------------------- */
void or_tri_rects(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                  int32_t* rects, int32_t* counts);
void or_tri_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                      const int32_t* rects, const int32_t* prefix,
                      int32_t* frag_pix, float* frag_attrs);
int64_t or_filter_valid(int64_t F, const int32_t* pix, const float* attrs,
                        int32_t* pix_out, float* attrs_out);
void or_depth_test(int B, int H, int W, int64_t F, const int32_t* frag_pix,
                   const float* frag_attrs, float* rast);
void or_cluster_mask(int64_t F, const int32_t* frag_pix, const float* frag_attrs,
                     const int32_t* prim2cluster, int H, int W, int S, int32_t* bitset);
void or_interpolate(int B, int H, int W, const float* rast, int C, const float* attr,
                    const int32_t* tri, double* image);
void or_interpolate_backward(int B, int H, int W, const float* rast, int C,
                             const float* d_image, const int32_t* tri, double* d_attr);
void or_dda_interpolate(int B, int H, int W, const float* rast, int C, const float* attr,
                        const int32_t* edges, double* image);
void or_dda_interpolate_backward(int B, int H, int W, const float* rast, int C,
                                 const float* d_image, const int32_t* edges, double* d_attr);

/* ---- antialias (antialias.cu, compact_utils.cu) ---------------------------------- */
void or_mark_edges(int H, int W, int B, int V, const float* pos, const int32_t* tri, int E,
                   const int32_t* edges, const int32_t* edge2tri, int32_t* prim_ids,
                   float* normals);
int64_t or_compact_ints(int64_t N, const int32_t* in, int32_t* out);
void or_aa_backward(int64_t F, const int32_t* frag_pix, const float* frag_attrs, int H, int W,
                    int S, const int32_t* bitset, const int32_t* target, int V,
                    const float* pos, int E, const int32_t* edges, const float* normals,
                    const int32_t* edge2cluster, double* d_pos, float kernel_radius, float rho,
                    double* frag_dc);

/* ---- bitset utils (bitset_utils.cu) ---------------------------------------------- */
void or_popcount(int64_t npix, int S, const int32_t* bitset, float* out);
void or_accumulate_rgb(int64_t npix, int S, const int32_t* bitset, const float* rgb, float* out);

/* ---- curves (curve_utils.cu) ----------------------------------------------------- */
void or_smooth_strands(int N, int V, const float* strands, const float* arclength,
                       double* out, float beta);
void or_skinning(int N, int V, const float* strands, const float* arclength,
                 const float* handles, const float* canonical, const float* R,
                 double* out, float beta);
void or_knn4(int64_t Nv, const float* x, int G, const float* g, int32_t* idx, float* d2);

#ifdef __cplusplus
}
#endif
#endif
