// Device-wide prefix sums and order-preserving stream compaction.
//
// Replaces the reference's thrust::inclusive_scan (dda.cu:111-115, rasterize.cu:77-81)
// and its block-local compaction with an atomic block base (rasterize.cu:280-365,
// compact_utils.cu:7-77), whose output order depends on block scheduling.  Here the
// order is the input order, and nothing synchronises with the host unless the caller
// asks for the count.  Reduce-then-scan in three launches: per-tile totals, a scan of
// the tile totals in one CTA, then a per-tile scan that adds the tile offset; an int32
// scan of at most 16,384 values runs in one CTA and one launch.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"
#include "scan.cuh"
#include "list.cuh"

namespace s2c {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ T warp_inclusive(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// exclusive scan of one value per thread over the block; returns the block total too
template <class T>
__device__ __forceinline__ T block_exclusive(T v, T* warp_buf, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T inc = warp_inclusive(v);
    if (lane == 31) warp_buf[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? warp_buf[lane] : T(0);
        const T wi = warp_inclusive(w);
        if (lane < nw) warp_buf[lane] = wi - w;
        if (lane == nw - 1) warp_buf[32] = wi;
    }
    __syncthreads();
    const T out = warp_buf[warp] + inc - v;
    total = warp_buf[32];
    __syncthreads();
    return out;
}

struct CountI32 {
    const int32_t* in;
    __device__ int64_t operator()(int64_t i) const { return in[i]; }
};
struct FlagFrag {
    const int32_t* pix;
    __device__ int64_t operator()(int64_t i) const { return pix[3 * i] >= 0 ? 1 : 0; }
};
struct FlagInt {
    const int32_t* in;
    __device__ int64_t operator()(int64_t i) const { return in[i] >= 0 ? 1 : 0; }
};

template <class F>
__global__ void __launch_bounds__(kScanThreads) tile_totals(F f, int64_t n, int64_t* sums) {
    __shared__ int64_t wb[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const int64_t i = base + (int64_t)j * kScanThreads + threadIdx.x;
        if (i < n) s += f(i);
    }
    int64_t tot;
    block_exclusive<int64_t>(s, wb, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// exclusive scan of the tile totals in place (one CTA), grand total to *total
__global__ void __launch_bounds__(1024) scan_totals(int64_t* sums, int64_t ntiles, int64_t* total) {
    __shared__ int64_t wb[33];
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = i < ntiles ? sums[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive<int64_t>(v, wb, tot);
        if (i < ntiles) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

// The whole inclusive int32 prefix of n <= kSmallScanMax values in one CTA (one launch
// instead of three); each thread owns up to kSmallScanItems consecutive values, so it
// writes only what it read and in == out works.
constexpr int kSmallScanThreads = 1024;
constexpr int kSmallScanItems = 16;
constexpr int64_t kSmallScanMax = (int64_t)kSmallScanThreads * kSmallScanItems;

__global__ void __launch_bounds__(kSmallScanThreads) scan_small_i32(const int32_t* in, int n, int32_t* out,
                                                                    int64_t* total) {
    __shared__ int64_t wb[33];
    const int per = (n + kSmallScanThreads - 1) / kSmallScanThreads;
    const int i0 = threadIdx.x * per;
    int32_t v[kSmallScanItems];
    int64_t s = 0;
#pragma unroll
    for (int j = 0; j < kSmallScanItems; ++j) {
        v[j] = (j < per && i0 + j < n) ? in[i0 + j] : 0;
        s += v[j];
    }
    int64_t tot;
    int64_t run = block_exclusive<int64_t>(s, wb, tot);
#pragma unroll
    for (int j = 0; j < kSmallScanItems; ++j) {
        run += v[j];
        if (j < per && i0 + j < n) out[i0 + j] = (int32_t)(uint32_t)(uint64_t)run;
    }
    if (threadIdx.x == 0) *total = tot;
}

// inclusive int32 prefix (wrapping like the reference's int scan)
__global__ void __launch_bounds__(kScanThreads) tile_scan_i32(const int32_t* in, int64_t n,
                                                              const int64_t* offs, int32_t* out) {
    __shared__ int64_t wb[33];
    __shared__ int32_t buf[kScanTile];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int j = 0; j < kScanItems; ++j) {
        const int64_t i = base + (int64_t)j * kScanThreads + threadIdx.x;
        buf[j * kScanThreads + threadIdx.x] = i < n ? in[i] : 0;
    }
    __syncthreads();
    int64_t s = 0;
    for (int j = 0; j < kScanItems; ++j) s += buf[threadIdx.x * kScanItems + j];
    int64_t tot;
    int64_t run = block_exclusive<int64_t>(s, wb, tot) + offs[blockIdx.x];
    for (int j = 0; j < kScanItems; ++j) {
        run += buf[threadIdx.x * kScanItems + j];
        buf[threadIdx.x * kScanItems + j] = (int32_t)(uint32_t)(uint64_t)run;
    }
    __syncthreads();
    for (int j = 0; j < kScanItems; ++j) {
        const int64_t i = base + (int64_t)j * kScanThreads + threadIdx.x;
        if (i < n) out[i] = buf[j * kScanThreads + threadIdx.x];
    }
}

template <class F, class Move>
__global__ void __launch_bounds__(kScanThreads) tile_scatter(F f, Move mv, int64_t n, const int64_t* offs) {
    __shared__ int64_t wb[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int flags = 0, s = 0;
    for (int j = 0; j < kScanItems; ++j) {
        const int64_t i = base + j;
        if (i < n && f(i)) { flags |= 1 << j; ++s; }
    }
    int64_t tot;
    int64_t pos = block_exclusive<int64_t>((int64_t)s, wb, tot) + offs[blockIdx.x];
    for (int j = 0; j < kScanItems; ++j)
        if (flags & (1 << j)) mv(base + j, pos++);
}

struct MoveFrag {
    const int32_t* pix; const float* attrs; int32_t* pix_out; float* attrs_out;
    __device__ void operator()(int64_t i, int64_t o) const {
        pix_out[3 * o] = pix[3 * i];
        pix_out[3 * o + 1] = pix[3 * i + 1];
        pix_out[3 * o + 2] = pix[3 * i + 2];
        reinterpret_cast<float4*>(attrs_out)[o] = reinterpret_cast<const float4*>(attrs)[i];
    }
};
struct MoveInt {
    const int32_t* in; int32_t* out;
    __device__ void operator()(int64_t i, int64_t o) const { out[o] = in[i]; }
};

int64_t scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

size_t scan_workspace_bytes(int64_t n) { return align_up((size_t)(scan_tiles(n) + 2) * sizeof(int64_t), 256); }

s2c_status inclusive_scan_i32(const int32_t* in, int64_t n, int32_t* out, void* ws, int64_t* d_total,
                              cudaStream_t st) {
    int64_t* sums = (int64_t*)ws;
    const int64_t nt = scan_tiles(n);
    if (n == 0) {
        cudaMemsetAsync(d_total, 0, sizeof(int64_t), st);
        return cuda_status(cudaGetLastError(), "scan: memset");
    }
    if (n <= kSmallScanMax) {
        scan_small_i32<<<1, kSmallScanThreads, 0, st>>>(in, (int)n, out, d_total);
        S2C_CHECK_LAUNCH("inclusive_scan_i32");
        return S2C_OK;
    }
    tile_totals<<<(unsigned)nt, kScanThreads, 0, st>>>(CountI32{in}, n, sums);
    scan_totals<<<1, 1024, 0, st>>>(sums, nt, d_total);
    tile_scan_i32<<<(unsigned)nt, kScanThreads, 0, st>>>(in, n, sums, out);
    S2C_CHECK_LAUNCH("inclusive_scan_i32");
    return S2C_OK;
}

s2c_status compact_fragments(const int32_t* pix, const float* attrs, int64_t n, int32_t* pix_out,
                             float* attrs_out, void* ws, int64_t* d_total, cudaStream_t st) {
    int64_t* sums = (int64_t*)ws;
    const int64_t nt = scan_tiles(n);
    if (n == 0) {
        cudaMemsetAsync(d_total, 0, sizeof(int64_t), st);
        return cuda_status(cudaGetLastError(), "compact: memset");
    }
    tile_totals<<<(unsigned)nt, kScanThreads, 0, st>>>(FlagFrag{pix}, n, sums);
    scan_totals<<<1, 1024, 0, st>>>(sums, nt, d_total);
    tile_scatter<<<(unsigned)nt, kScanThreads, 0, st>>>(FlagFrag{pix}, MoveFrag{pix, attrs, pix_out, attrs_out}, n, sums);
    S2C_CHECK_LAUNCH("compact_fragments");
    return S2C_OK;
}

s2c_status compact_ints(const int32_t* in, int64_t n, int32_t* out, void* ws, int64_t* d_total, cudaStream_t st) {
    int64_t* sums = (int64_t*)ws;
    const int64_t nt = scan_tiles(n);
    if (n == 0) {
        cudaMemsetAsync(d_total, 0, sizeof(int64_t), st);
        return cuda_status(cudaGetLastError(), "compact: memset");
    }
    tile_totals<<<(unsigned)nt, kScanThreads, 0, st>>>(FlagInt{in}, n, sums);
    scan_totals<<<1, 1024, 0, st>>>(sums, nt, d_total);
    tile_scatter<<<(unsigned)nt, kScanThreads, 0, st>>>(FlagInt{in}, MoveInt{in, out}, n, sums);
    S2C_CHECK_LAUNCH("compact_ints");
    return S2C_OK;
}

s2c_status read_count(const int64_t* d_total, int64_t* host, cudaStream_t st) {
    if (!host) return S2C_OK;
    cudaError_t e = cudaMemcpyAsync(host, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e, "reading a device count");
}

}  // namespace s2c

using namespace s2c;

namespace s2c {

__global__ void popc_words_kernel(int64_t n, const uint32_t* __restrict__ mask, int32_t* __restrict__ counts) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        counts[i] = __popc(mask[i]);
}

size_t list_carve(int64_t F, void* base, size_t cap, ListWs* w) {
    Carver cv(base, cap);
    ListWs r;
    const int64_t nw = std::max<int64_t>((F + 31) / 32, 1);
    r.mask = cv.take<uint32_t>(nw);
    r.wpre = cv.take<int32_t>(nw);
    r.total = cv.take<int64_t>(1);
    r.scan = cv.take<char>(scan_workspace_bytes(nw));
    if (w) *w = r;
    return cv.off;
}

s2c_status list_count(int64_t F, const ListWs& w, int64_t* num, cudaStream_t st) {
    const int64_t nw = (F + 31) / 32;
    if (nw > 0) {
        popc_words_kernel<<<grid_for(nw, 256, (int64_t)num_sms() * 8), 256, 0, st>>>(nw, w.mask, w.wpre);
        S2C_CHECK_LAUNCH("popc_words_kernel");
    }
    if (s2c_status s = inclusive_scan_i32(w.wpre, nw, w.wpre, w.scan, w.total, st)) return s;
    return read_count(w.total, num, st);
}

}  // namespace s2c

extern "C" size_t s2c_filter_valid_fragments_workspace_size(int64_t n) { return scan_workspace_bytes(n) + 256; }
extern "C" size_t s2c_compact_valid_ints_workspace_size(int64_t n) { return scan_workspace_bytes(n) + 256; }

extern "C" s2c_status s2c_filter_valid_fragments(int64_t num_frags, const int32_t* frag_pix,
                                                 const float* frag_attrs, int32_t* frag_pix_out,
                                                 float* frag_attrs_out, void* workspace,
                                                 size_t workspace_bytes, int64_t* num_valid,
                                                 s2c_stream stream) {
    S2C_REQUIRE(num_frags >= 0, "filter_valid_fragments: negative fragment count");
    S2C_REQUIRE(num_frags == 0 || (frag_pix && frag_attrs && frag_pix_out && frag_attrs_out),
                "filter_valid_fragments: null pointer");
    S2C_REQUIRE(((uintptr_t)frag_attrs & 15) == 0 && ((uintptr_t)frag_attrs_out & 15) == 0,
                "filter_valid_fragments: misaligned frag_attrs");
    if (workspace_bytes < s2c_filter_valid_fragments_workspace_size(num_frags) || !workspace) {
        set_error("filter_valid_fragments: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    int64_t* d_total = (int64_t*)((char*)workspace + scan_workspace_bytes(num_frags));
    s2c_status s = compact_fragments(frag_pix, frag_attrs, num_frags, frag_pix_out, frag_attrs_out, workspace,
                                     d_total, (cudaStream_t)stream);
    if (s) return s;
    return read_count(d_total, num_valid, (cudaStream_t)stream);
}

extern "C" s2c_status s2c_compact_valid_ints(int64_t n, const int32_t* input, int32_t* output, void* workspace,
                                             size_t workspace_bytes, int64_t* num_valid, s2c_stream stream) {
    S2C_REQUIRE(n >= 0, "compact_valid_ints: negative size");
    S2C_REQUIRE(n == 0 || (input && output), "compact_valid_ints: null pointer");
    if (workspace_bytes < s2c_compact_valid_ints_workspace_size(n) || !workspace) {
        set_error("compact_valid_ints: workspace too small");
        return S2C_ERR_WORKSPACE;
    }
    int64_t* d_total = (int64_t*)((char*)workspace + scan_workspace_bytes(n));
    s2c_status s = compact_ints(input, n, output, workspace, d_total, (cudaStream_t)stream);
    if (s) return s;
    return read_count(d_total, num_valid, (cudaStream_t)stream);
}
