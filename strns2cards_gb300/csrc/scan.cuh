// Device-wide scans and compaction shared by the raster entry points (scan.cu).
#pragma once
#include "common.cuh"

namespace s2c {
size_t scan_workspace_bytes(int64_t n);
// inclusive int32 prefix of in[0..n) into out (wrapping), total (int64) to *d_total
s2c_status inclusive_scan_i32(const int32_t* in, int64_t n, int32_t* out, void* ws, int64_t* d_total,
                              cudaStream_t st);
// keep fragments with pix[3i] >= 0, in order; kept count to *d_total
s2c_status compact_fragments(const int32_t* pix, const float* attrs, int64_t n, int32_t* pix_out,
                             float* attrs_out, void* ws, int64_t* d_total, cudaStream_t st);
s2c_status compact_ints(const int32_t* in, int64_t n, int32_t* out, void* ws, int64_t* d_total,
                        cudaStream_t st);
// copy a device count to the host and synchronise (no-op when host == nullptr)
s2c_status read_count(const int64_t* d_total, int64_t* host, cudaStream_t st);
}  // namespace s2c
