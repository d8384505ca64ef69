"""GB300-native strands-to-cards raster path: sm_103a CUDA kernels behind a C ABI.

The public ops keep the names and contracts of the reference package ``pystrns2cards``
so that ``import strns2cards_gb300 as s2c`` replaces ``import pystrns2cards as s2c``.
"""
from .antialias import (antialiased_cluster_bitset_grad, antialiased_cluster_bitset_loss,  # noqa: F401
                        mark_discontinuity_edges)
from .deform import CardLaplacian, LBSBinding, card_laplacian_smooth, lbs, vertex_adjacency  # noqa: F401
from .curve_utils import (align_wisp, align_wisps, align_wisps_packed, compute_aligned_strands,  # noqa: F401
                          compute_alignment_rotation, compute_arclength, compute_bishop_frame, minimal_rotation,
                          skinning, smooth_strands, strands_to_tube, tangent_frame)
from .bitset_utils import accumulate_bitset_rgb, cluster_iou, popcount_bitset, xor_error  # noqa: F401
from .dda import (DDAInterpolateAttributes, dda_cluster_bitset, dda_compute_fragments,  # noqa: F401
                  dda_interpolate_attributes)
from .mesh import build_edges_from_triangles, build_edges_from_triangles_device  # noqa: F401
from .texture import msaa_pattern, msaa_render, msaa_render_loop, resolve_patch  # noqa: F401
from .strands import load_strands, load_strands_arc_length, resample_strands_by_arclength  # noqa: F401
from .rasterize import (InterpolateTriangleAttributes, barycentric_derivatives, cluster_mask_from_fragments,  # noqa: F401
                        compute_fragments, depth_test, interpolate_triangle_attributes, rasterize,
                        rasterize_fused, rasterize_with_derivatives)
from . import _core  # noqa: F401
