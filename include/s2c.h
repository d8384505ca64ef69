/*
 * s2c.h -- C ABI of the GB300 strands-to-cards raster path (libs2c.so).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream, launches
 * sm_103a kernels on that stream and returns an s2c_status (never exits the process).
 * Outputs and scratch ("workspace") are allocated by the caller; each entry that needs
 * scratch has a *_workspace_size() query.  Entries that return a count to the host
 * (the reference's drop-in surface does) synchronise the stream; all others are
 * asynchronous.
 *
 * The "replaces" line of each entry names the reference interface it stands in for,
 * as a path inside the reference project (pystrns2cards/src/pystrns2cards.cpp is the
 * nanobind module `_core`; the launchers live in the *.cu files next to it).
 *
 * Layouts (all C-contiguous, little-endian):
 *   pos     float32 (B, V, 4)   homogeneous clip-space vertex positions, one set per view
 *   edges   int32   (E, 2)      vertex indices of line segments / mesh edges
 *   tri     int32   (T, 3)
 *   bitset  int32   (B, H, W, S), S = ceil(K / 32); cluster c is bit c % 32 of slot c / 32
 *   frag_pix int32 (F, 3) = (view, row, col); frag_attrs float32 (F, 4)
 */
#ifndef S2C_H
#define S2C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define S2C_API __attribute__((visibility("default")))
#else
#define S2C_API
#endif

typedef int s2c_status;
#define S2C_OK 0
#define S2C_ERR_INVALID 1     /* bad shape, size, pointer or argument               */
#define S2C_ERR_CUDA 2        /* a CUDA runtime call or kernel launch failed         */
#define S2C_ERR_WORKSPACE 3   /* caller workspace smaller than *_workspace_size()    */
#define S2C_ERR_TIMEOUT 4     /* a bounded device-side wait gave up                  */

/* a cudaStream_t; NULL = the legacy default stream */
typedef struct CUstream_st* s2c_stream;

S2C_API int s2c_version(void);
/* message of the last failed call on this host thread ("" if none) */
S2C_API const char* s2c_last_error(void);

/* ---------------------------------------------------------------------------------- *
 * DDA line raster                                                                     *
 * ---------------------------------------------------------------------------------- */

/* replaces: dda_compute_span (pystrns2cards.cpp:531-565; dda.cu:89-122).
 * Per primitive p (edge id edge_ids[p] = b*E + e, or p itself when edge_ids is NULL):
 * fragment count, (axis, slope) and (start_x, start_y, offset0, offset1); writes the
 * inclusive int32 prefix sum of the counts.  When num_frags != NULL the total is copied
 * to the host (stream synchronised), as the reference's return value. */
S2C_API size_t s2c_dda_compute_span_workspace_size(int64_t num_prims);
S2C_API s2c_status s2c_dda_compute_span(int64_t num_prims, const int32_t* edge_ids, int H, int W,
                                int B, int V, const float* pos, int E, const int32_t* edges,
                                int32_t* frag_prefix_sum, float* frag_slopes, float* frag_spans,
                                void* workspace, size_t workspace_bytes, int64_t* num_frags,
                                s2c_stream stream);

/* replaces: dda_compute_fragments (pystrns2cards.cpp:567-611; dda.cu:146-256).
 * frag_pix must be pre-filled with -1 (rejected fragments keep -1, as in the reference). */
S2C_API s2c_status s2c_dda_compute_fragments(int64_t num_prims, int64_t num_frags,
                                     const int32_t* frag_prefix_sum, const int32_t* edge_ids,
                                     const float* frag_slopes, const float* frag_spans, int H,
                                     int W, int B, int V, const float* pos, int E,
                                     const int32_t* edges, int32_t* frag_pix,
                                     float* frag_attrs, s2c_stream stream);

/* new: the compacted list -- what s2c_filter_valid_fragments leaves of
 * s2c_dda_compute_fragments' list, same order and values -- without the raw list (as
 * s2c_count_fragments / s2c_write_fragments for triangles): count after s2c_dda_compute_span
 * (num_steps = its count; *num_frags on the host, synchronising), then write on the same
 * stream with the same workspace (16-byte aligned). */
S2C_API size_t s2c_dda_count_fragments_workspace_size(int64_t num_steps);
S2C_API s2c_status s2c_dda_count_fragments(int64_t num_prims, int64_t num_steps, const int32_t* frag_prefix_sum,
                                           const int32_t* edge_ids, const float* frag_slopes,
                                           const float* frag_spans, int H, int W, int B, int V, const float* pos,
                                           int E, const int32_t* edges, void* workspace, size_t workspace_bytes,
                                           int64_t* num_frags, s2c_stream stream);
S2C_API s2c_status s2c_dda_write_fragments(int64_t num_prims, int64_t num_steps, const int32_t* frag_prefix_sum,
                                           const int32_t* edge_ids, const float* frag_slopes,
                                           const float* frag_spans, int H, int W, int B, int V, const float* pos,
                                           int E, const int32_t* edges, const void* workspace,
                                           size_t workspace_bytes, int32_t* frag_pix, float* frag_attrs,
                                           s2c_stream stream);

/* replaces: filter_valid_fragments (pystrns2cards.cpp:358-392; rasterize.cu:280-365).
 * Keeps fragments with frag_pix[i,0] >= 0 in their original order (the reference's order
 * depends on block scheduling); the kept count goes to *num_valid (host, synchronising). */
S2C_API size_t s2c_filter_valid_fragments_workspace_size(int64_t num_frags);
S2C_API s2c_status s2c_filter_valid_fragments(int64_t num_frags, const int32_t* frag_pix,
                                      const float* frag_attrs, int32_t* frag_pix_out,
                                      float* frag_attrs_out, void* workspace,
                                      size_t workspace_bytes, int64_t* num_valid,
                                      s2c_stream stream);

/* replaces: cluster_mask_from_fragments (pystrns2cards.cpp:440-478; rasterize.cu:474-520).
 * ORs bit prim2cluster[prim] of every fragment into a caller-zeroed bitset (B, H, W, S). */
S2C_API s2c_status s2c_cluster_mask_from_fragments(int64_t num_frags, const int32_t* frag_pix,
                                           const float* frag_attrs, const int32_t* prim2cluster,
                                           int64_t num_prims, int B, int H, int W, int S,
                                           int32_t* bitset, s2c_stream stream);

/* new (no single reference call; = dda_compute_fragments followed by
 * cluster_mask_from_fragments, as 3_fitting.py:254-261 uses them).
 * Rasterises every primitive straight into the bitset without a fragment list: segments
 * are binned into screen tiles, each tile's bitset is assembled in shared memory and
 * written once with coalesced stores.  The whole bitset (B, H, W, S) is overwritten.
 * edge_ids may be NULL (all B*E segments).  Bit-identical to the reference composition. */
S2C_API size_t s2c_dda_cluster_bitset_workspace_size(int64_t num_prims, int B, int H, int W, int S);
S2C_API s2c_status s2c_dda_cluster_bitset(int64_t num_prims, const int32_t* edge_ids, int H, int W,
                                  int B, int V, const float* pos, int E, const int32_t* edges,
                                  const int32_t* prim2cluster, int S, int32_t* bitset,
                                  void* workspace, size_t workspace_bytes, s2c_stream stream);
/* No counterpart in the reference.  s2c_dda_cluster_bitset for callers that cannot
 * allocate device memory (a plugin inside a host application that owns the device memory
 * pool and passes only input and output buffers, or a C caller with no allocator): the
 * scratch is a 32 MiB array inside libs2c.so that every GPU loading the library holds
 * until the process exits.  Problems whose s2c_dda_cluster_bitset_workspace_size()
 * exceeds 32 MiB are rejected with S2C_ERR_INVALID (about 1.4M segments at 1024x1024).
 * No cudaMalloc/cudaFree.  The first call on each device looks up the array's device
 * address (make it before any stream capture) and keeps it for the process: do not call
 * this entry after cudaDeviceReset (or after the primary context was released and made
 * again), where that address is no longer valid.  All calls share the array, so calls that
 * overlap on the GPU (different streams, or different host threads) race; serialise them.
 * s2c_dda_cluster_bitset_stats needs the workspace pointer and so is not available here.
 * Bad arguments are rejected on the host before any CUDA call, as for the entry above. */
S2C_API s2c_status s2c_dda_cluster_bitset_noalloc(int64_t num_prims, const int32_t* edge_ids, int H,
                                                  int W, int B, int V, const float* pos, int E,
                                                  const int32_t* edges, const int32_t* prim2cluster,
                                                  int S, int32_t* bitset, s2c_stream stream);
/* new (no single reference call; one iteration of the per-cluster fitting loop of
 * 3_fitting.py:381-406 for every cluster at once, in one persistent launch).  C clusters,
 * each framed at H x W with one cluster per view: strands strand_pos (C, Vs, 4) with a
 * shared edge list strand_edges (Es, 2) and edge_ids[i] = c * Es + e grouped by cluster,
 * cluster c owning edge_ids[cluster_offsets[c] .. cluster_offsets[c + 1]); cards card_pos
 * (C, Vc, 4), updated in place, sharing card_tri (Tc, 3), card_edges / card_edge2tri (Ec, 2)
 * and the Laplacian neighbour CSR of one card (lap_offsets (Vc + 1), lap_adj (nadj)).
 * With vert_offsets (C + 1) non-NULL the strand vertices are packed instead: cluster c's are
 * strand_pos rows vert_offsets[c] .. vert_offsets[c + 1] (Vs is then unused).
 * Per cluster: the strands' DDA coverage (exact, as dda_compute_fragments +
 * cluster_mask_from_fragments), the card raster's coverage (exact), the antialiased-bitset
 * gradient d_pos (FP64 sums), x, y -= d_pos * (step_scale / max |d_pos.xy|), then
 * laplacian_steps Jacobi steps p -= lam (p - mean of neighbours).  items (n_items, 2) lists
 * (cluster, chunk) work items in processing order with chunk segments each and
 * chunks_per_cluster (C) their counts; threads (128/256/512/1024), ctas_per_sm and aa_warp
 * (one warp rather than one thread per antialias fragment) shape the launch.  Limits:
 * H * ceil(W / 32) <= 16384, Vc <= 2048, Ec <= 8192.  The workspace is cleared on the
 * stream by each call; calls sharing one workspace must not overlap. */
S2C_API size_t s2c_fit_smem_bytes(int H, int W, int Vc, int Ec, int nadj);
S2C_API size_t s2c_fit_workspace_size(int C, int H, int W);
S2C_API s2c_status s2c_fit_iteration(int C, int H, int W, int Vs, const float* strand_pos,
                                     const int32_t* vert_offsets, int Es,
                                     const int32_t* strand_edges, const int32_t* edge_ids,
                                     const int32_t* cluster_offsets, int Vc, float* card_pos,
                                     int Tc, const int32_t* card_tri, int Ec,
                                     const int32_t* card_edges, const int32_t* card_edge2tri,
                                     const int32_t* lap_offsets, const int32_t* lap_adj, int nadj,
                                     const int32_t* items, int n_items, int chunk,
                                     const int32_t* chunks_per_cluster, float step_scale, float lam,
                                     int laplacian_steps, float kernel_radius, float rho,
                                     int threads, int ctas_per_sm, int aa_warp, void* workspace,
                                     size_t workspace_bytes, s2c_stream stream);

/* after a call on the same stream (synchronise first): how many primitives took the
 * global-atomic fallback because the workspace or a tile's record list was full */
S2C_API s2c_status s2c_dda_cluster_bitset_stats(const void* workspace, size_t workspace_bytes,
                                        int64_t* entries, int64_t* overflow_prims);

/* ---------------------------------------------------------------------------------- *
 * triangle rasterisation and attribute interpolation                                  *
 * ---------------------------------------------------------------------------------- */

/* replaces: compute_triangle_rects (pystrns2cards.cpp:245-281; rasterize.cu:9-88).
 * rects int32 (B*T, 4) = (h0, h_len, w0, w_len); prefix = inclusive scan of h_len*w_len;
 * total to *num_frags (host, synchronising) when non-NULL. */
S2C_API size_t s2c_compute_triangle_rects_workspace_size(int B, int T);
S2C_API s2c_status s2c_compute_triangle_rects(int H, int W, int B, int V, const float* pos, int T,
                                              const int32_t* tri, int32_t* rects, int32_t* prefix,
                                              void* workspace, size_t workspace_bytes,
                                              int64_t* num_frags, s2c_stream stream);

/* replaces: compute_fragments (pystrns2cards.cpp:283-326; rasterize.cu:90-195).
 * frag_pix pre-filled with -1; covered pixels get (b, y, x) and (b0, b1, z, t + 1). */
S2C_API s2c_status s2c_compute_fragments(int H, int W, int B, int V, const float* pos, int T,
                                         const int32_t* tri, const int32_t* prefix,
                                         const int32_t* rects, int64_t num_frags, int32_t* frag_pix,
                                         float* frag_attrs, s2c_stream stream);

/* new: the compacted fragment list -- what s2c_filter_valid_fragments leaves of
 * s2c_compute_fragments' list, same order and values -- without the raw list.
 * count_fragments (after s2c_compute_triangle_rects, num_bbox_pixels = its count) marks the
 * covered bounding-box pixels in the workspace (16-byte aligned, count_fragments_workspace_size
 * bytes) and returns their number in *num_frags (host; synchronises the stream);
 * write_fragments, on the same stream with the same workspace, writes them into
 * frag_pix (num_frags, 3) / frag_attrs (num_frags, 4, 16-byte aligned). */
S2C_API size_t s2c_count_fragments_workspace_size(int64_t num_bbox_pixels);
S2C_API s2c_status s2c_count_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                       const int32_t* prefix, const int32_t* rects, int64_t num_bbox_pixels,
                                       void* workspace, size_t workspace_bytes, int64_t* num_frags,
                                       s2c_stream stream);
S2C_API s2c_status s2c_write_fragments(int H, int W, int B, int V, const float* pos, int T, const int32_t* tri,
                                       const int32_t* prefix, const int32_t* rects, int64_t num_bbox_pixels,
                                       const void* workspace, size_t workspace_bytes, int32_t* frag_pix,
                                       float* frag_attrs, s2c_stream stream);

/* replaces: depth_test (pystrns2cards.cpp:328-356; rasterize.cu:198-278).
 * rast_out (B, H, W, 4) must be zeroed by the caller (as rasterize.py:55-95 does); pixels
 * with fragments get the attributes of the nearest one (ties: first in fragment order). */
S2C_API size_t s2c_depth_test_workspace_size(int B, int H, int W);
S2C_API s2c_status s2c_depth_test(int B, int H, int W, int64_t num_frags, const int32_t* frag_pix,
                                  const float* frag_attrs, float* rast_out, void* workspace,
                                  size_t workspace_bytes, s2c_stream stream);

/* new: compute_fragments + depth_test + cluster_mask_from_fragments in one pass without a
 * fragment list or host synchronisation (capturable in a CUDA graph).  rast (B, H, W, 4)
 * (nullable) equals depth_test's output (exact depth ties go to the lower triangle id);
 * bitset (B, H, W, S) (nullable; zeroed here) equals cluster_mask_from_fragments' for
 * tri2cluster (num_tri2cluster entries).  The workspace holds the B*H*W 64-bit depth
 * keys, the triangles' screen rectangles and the prefix of their areas (the work is split
 * evenly over the bbox pixels on the device). */
S2C_API size_t s2c_rasterize_fused_workspace_size(int B, int H, int W, int T);
/* new: the same pass writing cluster planes (B, 32 S, H, ceil(W / 32)) (zeroed here) instead
 * of the (B, H, W, S) bitset -- the layout the antialias windows and the per-cluster counts
 * read -- and rast (nullable). */
S2C_API s2c_status s2c_rasterize_fused_planes(int B, int H, int W, int V, const float* pos, int T,
                                              const int32_t* tri, const int32_t* tri2cluster,
                                              int num_tri2cluster, int S, uint32_t* planes, float* rast,
                                              void* workspace, size_t workspace_bytes, s2c_stream stream);
/* new: the same pass ORing the cards' cluster bits onto planes the caller keeps (not cleared
 * here; they must hold zeros wherever this pass can set a bit, e.g. after
 * s2c_planes_clear_rects with the previous pass's rectangles), and writing cluster_rects
 * (B, 32 S, 4) int32, 16-byte aligned: per (view, plane) rows [y0, y1) x plane words
 * [q0, q1) holding every bit it can set (the union of the cluster's triangle rectangles;
 * empty = (H, 0, ceil(W / 32), 0)).  A fitting loop then clears and counts only those
 * rectangles instead of whole planes. */
S2C_API s2c_status s2c_rasterize_fused_planes_onto(int B, int H, int W, int V, const float* pos, int T,
                                                   const int32_t* tri, const int32_t* tri2cluster,
                                                   int num_tri2cluster, int S, uint32_t* planes,
                                                   int32_t* cluster_rects, void* workspace,
                                                   size_t workspace_bytes, s2c_stream stream);
S2C_API s2c_status s2c_rasterize_fused(int B, int H, int W, int V, const float* pos, int T, const int32_t* tri,
                                       const int32_t* tri2cluster, int num_tri2cluster, int S, int32_t* bitset,
                                       float* rast, void* workspace, size_t workspace_bytes, s2c_stream stream);

/* new: resolve of a software-MSAA render (texture_utils.py:189-226): rast (S, H, W, 4) of S
 * jittered rasterisations of one mesh; per pixel, in sample order, acc (H, W, C) += the
 * interpolated attribute (as s2c_interpolate_triangle_attributes) * valid, count (H, W) +=
 * valid, alpha (H, W) += weights[i] * valid, valid = rast.w > 0.  C <= 8. */
S2C_API s2c_status s2c_msaa_resolve(int S, int H, int W, int C, const float* rast, int V, const float* attr, int T,
                                    const int32_t* tri, const float* weights, float* acc, float* count,
                                    float* alpha, s2c_stream stream);

/* new: d(b0, b1)/d(x, y) in pixel units, rast_db (B, H, W, 4) = (db0/dx, db0/dy, db1/dx,
 * db1/dy), from the clip-space edge functions of the forward (rasterize.cu:144-156) for the
 * triangle id in rast (B, H, W, 4); 0 where rast is empty.  The reference has no such output. */
S2C_API s2c_status s2c_barycentric_derivatives(int B, int H, int W, int V, const float* pos, int T,
                                               const int32_t* tri, const float* rast, float* rast_db,
                                               s2c_stream stream);

/* replaces: interpolate_triangle_attributes (pystrns2cards.cpp:394-415; rasterize.cu:367-455).
 * image (B, H, W, C) pre-zeroed by the caller. */
S2C_API s2c_status s2c_interpolate_triangle_attributes(int B, int H, int W, int C, const float* rast,
                                                       int V, const float* attr, int T,
                                                       const int32_t* tri, float* image,
                                                       s2c_stream stream);

/* replaces: backward_interpolate_triangle_attributes (pystrns2cards.cpp:417-438;
 * rasterize.cu:402-472).  d_attr (V, C) += sum over pixels of b_i * grad.  acc64: NULL ->
 * float atomics straight into d_attr (the reference's arithmetic); else a caller buffer of
 * V*C doubles (8-byte aligned, cleared here): the exact FP32 products are summed in FP64
 * and each sum is rounded once into d_attr. */
S2C_API s2c_status s2c_backward_interpolate_triangle_attributes(int B, int H, int W, int C,
                                                                const float* rast,
                                                                const float* d_image, int T,
                                                                const int32_t* tri, int V,
                                                                float* d_attr, double* acc64,
                                                                s2c_stream stream);

/* replaces: dda_interpolate_attributes (pystrns2cards.cpp:613-647; dda.cu:258-298) */
S2C_API s2c_status s2c_dda_interpolate_attributes(int B, int H, int W, int C, const float* rast,
                                                  int V, const float* attr, int E,
                                                  const int32_t* edges, float* image,
                                                  s2c_stream stream);

/* replaces: backward_dda_interpolate_attributes (pystrns2cards.cpp:649-680; dda.cu:300-342).
 * acc64 as for s2c_backward_interpolate_triangle_attributes. */
S2C_API s2c_status s2c_backward_dda_interpolate_attributes(int B, int H, int W, int C,
                                                           const float* rast, const float* d_image,
                                                           int E, const int32_t* edges, int V,
                                                           float* d_attr, double* acc64,
                                                           s2c_stream stream);

/* ---------------------------------------------------------------------------------- *
 * stream compaction                                                                   *
 * ---------------------------------------------------------------------------------- */

/* replaces: compact_valid_ints (pystrns2cards.cpp:774-786; compact_utils.cu:54-77).
 * Order-preserving; count to *num_valid (host, synchronising). */
S2C_API size_t s2c_compact_valid_ints_workspace_size(int64_t n);
S2C_API s2c_status s2c_compact_valid_ints(int64_t n, const int32_t* input, int32_t* output,
                                  void* workspace, size_t workspace_bytes, int64_t* num_valid,
                                  s2c_stream stream);

/* ---------------------------------------------------------------------------------- *
 * bitset utilities                                                                    *
 * ---------------------------------------------------------------------------------- */

/* new: cluster planes of a bitset: planes (B, 32 S, H, ceil(W / 32)) uint32, bit (x & 31) of
 * word x >> 5 in row y of plane c = bit c of pixel (y, x).  A window of one cluster is then
 * a few contiguous words per row instead of one 32-byte sector per pixel. */
S2C_API size_t s2c_bitset_planes_size(int B, int H, int W, int S);
S2C_API s2c_status s2c_bitset_to_planes(int B, int H, int W, int S, const int32_t* bitset, uint32_t* planes,
                                        s2c_stream stream);

/* replaces: popcount_bitset (pystrns2cards.cpp:507-529; bitset_utils.cu:37-52,392-404) */
S2C_API s2c_status s2c_popcount_bitset(int64_t num_pixels, int S, const int32_t* bitset,
                               float* count_image, s2c_stream stream);

/* replaces: accumulate_bitset_rgb (pystrns2cards.cpp:480-505; bitset_utils.cu:6-35,376-390) */
S2C_API s2c_status s2c_accumulate_bitset_rgb(int64_t num_pixels, int S, const int32_t* bitset,
                                     int num_clusters, const float* cluster_rgb,
                                     float* accum_color, s2c_stream stream);

/* new: the XOR-popcount loss of antialias.py:124-126 (popcount_bitset(a ^ b).sum()) in
 * one pass; *total (device uint64) = sum over nwords int32 words of popc(a ^ b). */
S2C_API s2c_status s2c_xor_popcount(int64_t nwords, const int32_t* a, const int32_t* b,
                                    uint64_t* total, s2c_stream stream);

/* new: per-cluster pixel counts for the per-card bitset IoU: inter[c] = #pixels with bit c
 * set in both bitsets, uni[c] = #pixels with bit c set in either (device uint64, K each). */
S2C_API s2c_status s2c_cluster_iou_counts(int64_t num_pixels, int S, int K, const int32_t* a,
                                          const int32_t* b, uint64_t* inter, uint64_t* uni,
                                          s2c_stream stream);

/* new: per-cluster counts from cluster planes of two bitsets (as s2c_cluster_iou_counts). */
S2C_API s2c_status s2c_cluster_iou_counts_planes(int B, int H, int W, int S, int K, const uint32_t* a,
                                                 const uint32_t* b, uint64_t* inter, uint64_t* uni,
                                                 s2c_stream stream);

/* new: plane rectangles (B, 32 S, 4) int32 (y0, y1, q0, q1), 16-byte aligned: rows
 * [y0, y1) x plane words [q0, q1) of each (view, plane), clamped to the plane; y0 >= y1 or
 * q0 >= q1 is empty.  clear_rects zeroes each plane's rectangle; bounds writes the smallest
 * rectangle holding every non-zero word of each plane (empty = (H, 0, ceil(W / 32), 0)). */
S2C_API s2c_status s2c_planes_clear_rects(int B, int H, int W, int S, uint32_t* planes, const int32_t* rects,
                                          s2c_stream stream);
S2C_API s2c_status s2c_planes_bounds(int B, int H, int W, int S, const uint32_t* planes, int32_t* rects,
                                     s2c_stream stream);
/* new: s2c_cluster_iou_counts_planes counting only inside the bounding rectangle of each
 * plane's rects_a and rects_b rectangles -- exact when every set bit of a (b) lies inside its
 * rects_a (rects_b) rectangle -- and *xor_total (nullable, device uint64) = the XOR-popcount
 * loss over all 32 S planes (sum of union - inter), in the same pass. */
S2C_API s2c_status s2c_cluster_iou_counts_planes_rects(int B, int H, int W, int S, int K, const uint32_t* a,
                                                       const uint32_t* b, const int32_t* rects_a,
                                                       const int32_t* rects_b, uint64_t* inter, uint64_t* uni,
                                                       uint64_t* xor_total, s2c_stream stream);

/* ---------------------------------------------------------------------------------- *
 * antialiased cluster bitset loss                                                     *
 * ---------------------------------------------------------------------------------- */

/* replaces: mark_discontinuity_edges (pystrns2cards.cpp:682-715; antialias.cu:38-119).
 * prim_ids (B*E) pre-filled with -1 and normals (B*E, 2) zeroed by the caller; silhouette
 * and boundary edges get prim_ids[b*E+e] = b*E+e and an oriented unit normal. */
S2C_API s2c_status s2c_mark_discontinuity_edges(int H, int W, int B, int V, const float* pos, int T,
                                                const int32_t* tri, int E, const int32_t* edges,
                                                const int32_t* edge2tri, int32_t* prim_ids,
                                                float* normals, s2c_stream stream);

/* replaces: backward_antialiased_cluster_bitset (pystrns2cards.cpp:717-772; antialias.cu:121-317).
 * d_pos (B, V, 4) accumulated (x, y, w components) from the silhouette-edge fragments. */
S2C_API s2c_status s2c_backward_antialiased_cluster_bitset(
    int64_t num_frags, const int32_t* frag_pix, const float* frag_attrs, int B, int H, int W, int S,
    const int32_t* bitset, const int32_t* target, int V, const float* pos, int E,
    const int32_t* edges, const float* normals, const int32_t* edge2cluster, float* d_pos,
    float kernel_radius, float rho, s2c_stream stream);

/* new: the same gradient with each fragment's contribution formed and summed in FP64 in a
 * caller workspace (B*V*3 doubles), then added once into d_pos: d_pos is then the
 * correctly-rounded float of a (nearly) exact sum, independent of scheduling, instead of a
 * float-atomic sum whose cancellation error depends on it. */
S2C_API size_t s2c_backward_antialiased_cluster_bitset_workspace_size(int B, int V);
S2C_API s2c_status s2c_backward_antialiased_cluster_bitset_f64(
    int64_t num_frags, const int32_t* frag_pix, const float* frag_attrs, int B, int H, int W, int S,
    const int32_t* bitset, const int32_t* target, int V, const float* pos, int E,
    const int32_t* edges, const float* normals, const int32_t* edge2cluster, float* d_pos,
    float kernel_radius, float rho, void* workspace, size_t workspace_bytes, s2c_stream stream);

/* new: the whole gradient of antialias.py:100-122 in one pass -- the silhouette test, the
 * DDA walk of each marked edge and every fragment's window, fused per (view, edge), with no
 * fragment list and no host synchronisation (capturable in a CUDA graph).  Same
 * contributions as mark_discontinuity_edges + dda_compute_fragments + the backward above;
 * d_pos (B, V, 4) accumulated.  The workspace holds the FP64 accumulator (B*V*3 doubles)
 * and the cluster planes of both bitsets (see s2c_bitset_to_planes), read by the windows;
 * it must be 16-byte aligned.  At most 2^32 - 1 silhouette fragments per call. */
S2C_API size_t s2c_antialiased_cluster_bitset_grad_workspace_size(int B, int V, int H, int W, int S, int E);
S2C_API s2c_status s2c_antialiased_cluster_bitset_grad(
    int B, int H, int W, int S, const int32_t* bitset, const int32_t* target, int V, const float* pos, int T,
    const int32_t* tri, int E, const int32_t* edges, const int32_t* edge2tri, const int32_t* edge2cluster,
    float* d_pos, float kernel_radius, float rho, void* workspace, size_t workspace_bytes, s2c_stream stream);

/* new: the same from cluster planes the caller keeps (e.g. the target's, built once per fit);
 * workspace (16-byte aligned): the FP64 accumulator (B*V*3 doubles), per-(view, edge) work
 * counts and an 80-byte record per silhouette (view, edge) (end points, span, normal). */
S2C_API size_t s2c_antialiased_cluster_bitset_grad_planes_workspace_size(int B, int V, int E);
S2C_API s2c_status s2c_antialiased_cluster_bitset_grad_planes(
    int B, int H, int W, int S, const uint32_t* bitset_planes, const uint32_t* target_planes, int V,
    const float* pos, int T, const int32_t* tri, int E, const int32_t* edges, const int32_t* edge2tri,
    const int32_t* edge2cluster, float* d_pos, float kernel_radius, float rho, void* workspace,
    size_t workspace_bytes, s2c_stream stream);

/* ---------------------------------------------------------------------------------- *
 * strand curves                                                                       *
 * ---------------------------------------------------------------------------------- */

/* new: cumulative arclength of each strand, arclength[s, 0] = 0 and
 * arclength[s, i] = sum_{k<=i} |x[s,k] - x[s,k-1]| (curve_utils.py:167-180 computes the same
 * with torch.norm + torch.cumsum). strands (N, V, 3), arclength (N, V). */
S2C_API s2c_status s2c_compute_arclength(int N, int V, const float* strands, float* arclength,
                                         s2c_stream stream);

/* replaces: smooth_strands (pystrns2cards.cpp:841-872; curve_utils.cu:24-68,135-147).
 * out[s, i] = sum_j w_ij x[s, j] / sum_j w_ij over |a_i - a_j| <= 3 beta,
 * w_ij = exp(-(a_i - a_j)^2 / beta^2); points whose weight sum is <= 1e-6 are written 0
 * (the reference leaves them at the zero its caller filled in).  arclength may be NULL:
 * it is then computed in the kernel as s2c_compute_arclength does. */
S2C_API s2c_status s2c_smooth_strands(int N, int V, const float* strands, const float* arclength,
                                      float* smoothed_strands, float beta, s2c_stream stream);

/* replaces: skinning (pystrns2cards.cpp:873-915; curve_utils.cu:70-131,149-166).
 * out[s, i] = sum_j w_ij (R_j (x_i - h_j) + c_j) / sum_j w_ij with the weights of
 * s2c_smooth_strands; out = x where the weight sum is <= 1e-8.  R (N, V, 3, 3) row-major.
 * arclength may be NULL (computed in the kernel). */
S2C_API s2c_status s2c_skinning(int N, int V, const float* strands, const float* arclength,
                                const float* handle_strands, const float* canonical_handles,
                                const float* R, float* skinned_strands, float beta,
                                s2c_stream stream);

/* replaces: compute_bishop_frame, compute_alignment_rotation, compute_aligned_strands
 * (curve_utils.py:104-165, 273-308, 243-271), one thread per strand, FP32.
 * strands (N, V, 3).  Every output may be NULL:
 *   T, Nrm, Bin (N, V, 3): the double-reflection rotation-minimising frame, started from
 *     tangent_frame of the root tangent (curve_utils.py:76-102);
 *   R (N, V, 3, 3) row-major: [t_dst n_dst b_dst][T N B]^T, n_dst, b_dst the root frame
 *     turned by the minimal rotation of the root tangent onto t_dst;
 *   canon (N, V, 3): arclength * t_dst + root, the roots taken from `roots` (one per strand,
 *     roots_stride floats apart: 3 for an (N, 3) array, 3V for the first points of an
 *     (N, V, 3) array) or, when roots is NULL, from the strands themselves.
 * t_dst: 3 floats in HOST memory (needed for R and canon). */
S2C_API s2c_status s2c_strand_frames(int N, int V, const float* strands, const float* t_dst, float* T,
                                     float* Nrm, float* Bin, float* R, const float* roots,
                                     int64_t roots_stride, float* canon, s2c_stream stream);

/* replaces: the per-wisp loop of align_wisps (curve_utils.py:521-568): one CTA per wisp.
 * Wisp w holds strands offsets[w] .. offsets[w+1]-1 of strands (num_strands, V, 3), V >= 2.
 * centre[w] = mean root; longest[w] = the strand of greatest polyline length (first on
 * ties); the least-variance axis of the centred roots (FP32 second moment and a Jacobi
 * eigen-solve, in place of the host SVD; identity axes below 3 strands) and the longest
 * strand's view and down directions give the source frame; R_global[w] (3x3 row-major) =
 * [t_dst n_dst b_dst][T_src N_src B_src]^T.  An empty or out-of-range wisp gets the
 * identity, centre 0 and longest -1.  t_dst, n_dst, b_dst: 3 floats each in HOST memory. */
S2C_API s2c_status s2c_wisp_frames(int num_wisps, const int32_t* offsets, int64_t num_strands, int V,
                                   const float* strands, const float* t_dst, const float* n_dst,
                                   const float* b_dst, float* R_global, float* centre, int32_t* longest,
                                   s2c_stream stream);

/* new: a_out = R_global[w] (a - centre[w]) and b_out likewise for every point of every strand,
 * w the wisp whose range offsets[w] .. offsets[w+1]-1 holds the strand (offsets as for
 * s2c_wisp_frames, non-decreasing); a strand of no wisp is copied unchanged
 * (curve_utils.py:567-568 rotate the strands and the handle strands of each wisp). */
S2C_API s2c_status s2c_wisp_rotate(int num_wisps, const int32_t* offsets, int64_t num_strands, int V,
                                   const float* R_global, const float* centre, const float* a,
                                   const float* b, float* a_out, float* b_out, s2c_stream stream);

/* replaces: the rest of align_wisps after its per-wisp loop (curve_utils.py:487-606), fused:
 * per strand, handles = smooth_strands(strands, beta) (written out: align_wisps returns it),
 * then the strand and its handle turned into its wisp's frame as s2c_wisp_rotate does, the
 * handle's frames, alignment rotations and canonical handles (roots: the turned strand's
 * first point) as s2c_strand_frames does, and the turned strand skinned to them as
 * s2c_skinning does -- the same results bit for bit, with the intermediates kept in shared
 * memory.  Needs 2 <= V <= s2c_align_strands_max_points(); t_dst: 3 floats in HOST memory. */
S2C_API int s2c_align_strands_max_points(void);
S2C_API s2c_status s2c_align_strands(int64_t num_strands, int V, const float* strands, int num_wisps,
                                     const int32_t* offsets, const float* R_global, const float* centre,
                                     const float* t_dst, float beta, float* handles, float* aligned,
                                     s2c_stream stream);

/* replaces: load_strands (pystrns2cards.cpp:788-816; hair_loader.cpp:15-259).  Host.
 * Reads a .bin, .data (USC) or .hair (CY-HAIR / ZJU) file; *handle receives the strands
 * with at least two points (counts in *num_strands, total points in *num_points), to be
 * copied out and released by s2c_strands_take.  An unopenable file gives no strands (as
 * the reference); a truncated one is S2C_ERR_INVALID. */
S2C_API s2c_status s2c_load_strands(const char* path, void** handle, int64_t* num_strands, int64_t* num_points);
S2C_API s2c_status s2c_strands_take(void* handle, int32_t* num_samples, float* points);

/* replaces: resample_strands_by_arclength (pystrns2cards.cpp:818-839; hair_loader.cpp:261-307).
 * Host: points (sum(num_samples), 3) -> out (num_strands, target, 3), the reference's FP32
 * operations; strands need at least 2 points. */
S2C_API s2c_status s2c_resample_strands_by_arclength_host(int num_strands, const int32_t* num_samples,
                                                         const float* points, int target, float* out);

/* new: the same on the device, one thread per strand with the same FP32 operations (results
 * identical to the host version).  Strands with fewer than 2 points, or counts that
 * overrun num_points, give NaN rows. */
S2C_API size_t s2c_resample_strands_workspace_size(int num_strands, int64_t num_points);
S2C_API s2c_status s2c_resample_strands_by_arclength(int num_strands, const int32_t* num_samples,
                                                     const float* points, int64_t num_points, int target,
                                                     float* out, void* workspace, size_t workspace_bytes,
                                                     s2c_stream stream);

/* ---------------------------------------------------------------------------------- *
 * card mesh topology (host)                                                           *
 * ---------------------------------------------------------------------------------- */

/* replaces: build_edges_from_triangles (pystrns2cards.cpp:208-243; mesh_utils.cpp:36-95).
 * Host memory.  Unique undirected edges stored (min, max), sorted by (min, max) -- the
 * reference emits them in std::unordered_map order, which is implementation-defined --
 * and per edge the first two triangles that contain it (-1 where there is none).
 * edges and edge2tri hold 3*T rows; *num_edges receives the count. */
S2C_API s2c_status s2c_build_edges_from_triangles(int T, const int32_t* tri, int32_t* edges,
                                                  int32_t* edge2tri, int64_t* num_edges);

/* new: the same on the device, with the same edges in the same order and the same
 * edge2tri (deterministic: buckets per min vertex, each ordered by (max vertex, half-edge)).
 * tri (T, 3) device; edges and edge2tri hold 3*T rows; *num_edges (device int64) receives
 * the edge count and *num_bad (device int32) the half-edges left out for a vertex outside
 * [0, num_verts).  No host synchronisation. */
S2C_API size_t s2c_build_edges_device_workspace_size(int T, int num_verts);
S2C_API s2c_status s2c_build_edges_device(int T, const int32_t* tri, int num_verts, int32_t* edges,
                                          int32_t* edge2tri, int64_t* num_edges, int32_t* num_bad,
                                          void* workspace, size_t workspace_bytes, s2c_stream stream);

/* new: host.  CSR vertex adjacency of an undirected edge list (the uniform Laplacian's
 * A of optimizer.py:70-99): neighbours of v in edge order, offsets (num_verts + 1),
 * adj (2 E); *num_adj receives the count. */
S2C_API s2c_status s2c_build_vertex_adjacency(int num_verts, int E, const int32_t* edges, int32_t* offsets,
                                              int32_t* adj, int64_t* num_adj);

/* ---------------------------------------------------------------------------------- *
 * card deformation                                                                    *
 * ---------------------------------------------------------------------------------- */

/* new: Laplacian smoothing of card vertices, p <- p - lam * (p - mean of neighbours),
 * `steps` Jacobi steps.  The reference has no kernel for it; it builds L = D - A of the
 * card edges (optimizer.py:70-99) as preconditioner and regulariser (3_fitting.py:347-359).
 * All cards share one topology: CSR adjacency (adj_offsets (verts_per_card + 1),
 * adj (num_adj) local vertex ids); vertices (num_cards * verts_per_card, 3).  In place
 * allowed.  A vertex without neighbours keeps its position. */
S2C_API s2c_status s2c_card_laplacian_smooth(int num_cards, int verts_per_card, const int32_t* adj_offsets,
                                             const int32_t* adj, int num_adj, const float* verts_in,
                                             float* verts_out, float lam, int steps, s2c_stream stream);

/* new: binding of strand vertices x (Nv, 3) to their 4 nearest guides (G, 3): idx (Nv, 4)
 * (-1 where fewer than 4 guides exist), w (Nv, 4) = softmax(-d^2 / tau) over them, and the
 * inverse lists (CSR over guides: list_offsets (G + 1), list_entries (4 Nv) = v * 4 + slot,
 * ascending).  Distances are FP32 (dx^2 + dy^2) + dz^2; ties go to the lower guide index. */
S2C_API size_t s2c_lbs_bind_workspace_size(int64_t num_verts, int num_guides);
S2C_API s2c_status s2c_lbs_bind(int64_t num_verts, const float* x, int num_guides, const float* guides,
                                float tau, int32_t* idx, float* w, int32_t* list_offsets,
                                int32_t* list_entries, void* workspace, size_t workspace_bytes,
                                s2c_stream stream);

/* new: y = sum_k w_k (A_k x + t_k) with M (G, 3, 4) = [A | t] per guide. */
S2C_API s2c_status s2c_lbs_forward(int64_t num_verts, const float* x, const int32_t* idx, const float* w,
                                   int num_guides, const float* M, float* y, s2c_stream stream);

/* new: gradients of the forward for grad_y (Nv, 3): grad_M (G, 3, 4) (overwritten; per-guide
 * sums in the bind's list order) and, if non-NULL, grad_x (Nv, 3) = sum_k w_k A_k^T grad_y
 * (weights held at their bound values).  Either output may be NULL. */
S2C_API s2c_status s2c_lbs_backward(int64_t num_verts, const float* x, const int32_t* idx, const float* w,
                                    int num_guides, const float* M, const int32_t* list_offsets,
                                    const int32_t* list_entries, const float* grad_y, float* grad_M,
                                    float* grad_x, s2c_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* S2C_H */
