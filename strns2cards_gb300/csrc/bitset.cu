// Per-pixel bitset reductions (the reference's bitset_utils.cu) and bitset comparisons.
#include <algorithm>

#include "common.cuh"

namespace s2c {

// bitset_utils.cu:37-52; one thread per pixel, 16-byte loads when S % 4 == 0
// Per-pixel passes over a (npix, S) bitset.  A thread owns a pixel, but a pixel's words are
// 4 S bytes apart from its neighbours', so the CTA first stages 128 pixels x 16 slots
// through shared memory with 16-byte loads (every sector read whole), then each thread
// walks its pixel's words there in slot order (row stride 17 words: conflict-free).
constexpr int kBitsPix = 128, kBitsChunk = 16, kBitsRow = kBitsChunk + 1;

__device__ __forceinline__ void stage_bits(int64_t npix, int S, const int32_t* __restrict__ bits, int64_t p0, int s0,
                                           int n, bool vec, uint32_t* __restrict__ tile) {
    if (vec) {   // S % 4 == 0, 16-byte aligned: n / 4 int4 per pixel
        const int q = n >> 2;
        for (int i = threadIdx.x; i < kBitsPix * q; i += blockDim.x) {
            const int px = i / q, k = i - px * q;
            const int64_t p = p0 + px;
            int4 v = make_int4(0, 0, 0, 0);
            if (p < npix) v = __ldcs((const int4*)(bits + p * S + s0) + k);
            uint32_t* d = tile + px * kBitsRow + 4 * k;
            d[0] = (uint32_t)v.x;
            d[1] = (uint32_t)v.y;
            d[2] = (uint32_t)v.z;
            d[3] = (uint32_t)v.w;
        }
    } else {
        for (int i = threadIdx.x; i < kBitsPix * n; i += blockDim.x) {
            const int px = i / n, k = i - px * n;
            const int64_t p = p0 + px;
            tile[px * kBitsRow + k] = p < npix ? (uint32_t)__ldg(bits + p * S + s0 + k) : 0u;
        }
    }
}

__global__ void __launch_bounds__(kBitsPix) popcount_kernel(int64_t npix, int S, const int32_t* __restrict__ bits,
                                                            float* __restrict__ out) {
    __shared__ uint32_t tile[kBitsPix * kBitsRow];
    const int64_t p0 = (int64_t)blockIdx.x * kBitsPix;
    const bool vec = (S & 3) == 0 && ((uintptr_t)bits & 15) == 0;
    int n = 0;
    for (int s0 = 0; s0 < S; s0 += kBitsChunk) {
        const int m = min(kBitsChunk, S - s0);
        __syncthreads();
        stage_bits(npix, S, bits, p0, s0, m, vec, tile);
        __syncthreads();
        const uint32_t* row = tile + threadIdx.x * kBitsRow;
        for (int j = 0; j < m; ++j) n += __popc(row[j]);
    }
    const int64_t p = p0 + threadIdx.x;
    if (p < npix) out[p] = (float)n;
}

// bitset_utils.cu:6-35: clusters are visited in increasing id order, the same float
// summation order as the reference, so the sums are bit-identical.  Each thread walks its
// pixel's set bits in one flat loop (a nested word / bit loop would run, per word, as long
// as the lane with the most bits in that word: 0.75 -> 0.36 ms for popcount + colours of a
// 256 MiB bitset with 5 % of the words set).  Measured and not kept: threads taking pixels
// from a per-CTA counter (0.50 ms).
__global__ void __launch_bounds__(kBitsPix) accumulate_rgb_kernel(int64_t npix, int S, const int32_t* __restrict__ bits,
                                                                  int K, const float* __restrict__ rgb,
                                                                  float* __restrict__ out) {
    __shared__ uint32_t tile[kBitsPix * kBitsRow];
    const int64_t p0 = (int64_t)blockIdx.x * kBitsPix;
    const bool vec = (S & 3) == 0 && ((uintptr_t)bits & 15) == 0;
    float r = 0.f, g = 0.f, b = 0.f;
    for (int s0 = 0; s0 < S; s0 += kBitsChunk) {
        const int m = min(kBitsChunk, S - s0);
        __syncthreads();
        stage_bits(npix, S, bits, p0, s0, m, vec, tile);
        __syncthreads();
        const uint32_t* row = tile + threadIdx.x * kBitsRow;
        uint32_t nz = 0;
        for (int j = 0; j < m; ++j) nz |= (uint32_t)(row[j] != 0u) << j;
        uint32_t w = 0;
        int base = 0;
        while (nz | w) {
            if (!w) {
                const int j = __ffs(nz) - 1;
                nz &= nz - 1;
                w = row[j];
                base = (s0 + j) * 32;
                continue;
            }
            const int c = base + __ffs(w) - 1;
            w &= w - 1;
            if (c >= K) continue;
            r = __fadd_rn(r, __ldg(rgb + 3 * c));
            g = __fadd_rn(g, __ldg(rgb + 3 * c + 1));
            b = __fadd_rn(b, __ldg(rgb + 3 * c + 2));
        }
    }
    const int64_t p = p0 + threadIdx.x;
    if (p < npix) {
        out[3 * p] = r;
        out[3 * p + 1] = g;
        out[3 * p + 2] = b;
    }
}

// sum over all words of popc(a ^ b): the XOR-popcount loss of antialias.py:124-126 in one
// pass (the reference materialises a ^ b, a float popcount image and its sum)
__global__ void __launch_bounds__(256) xor_popcount_kernel(int64_t nwords, const int32_t* __restrict__ a,
                                                           const int32_t* __restrict__ b,
                                                           unsigned long long* __restrict__ total) {
    const int64_t n4 = nwords >> 2;
    const int4* a4 = reinterpret_cast<const int4*>(a);
    const int4* b4 = reinterpret_cast<const int4*>(b);
    unsigned long long s = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const int4 x = __ldcs(a4 + i), y = __ldcs(b4 + i);
        s += __popc(x.x ^ y.x) + __popc(x.y ^ y.y) + __popc(x.z ^ y.z) + __popc(x.w ^ y.w);
    }
    for (int64_t i = (n4 << 2) + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += stride)
        s += __popc(a[i] ^ b[i]);
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ unsigned long long ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
        atomicAdd(total, t);
    }
}

// per-cluster pixel counts of a & b and a | b (per-card IoU = inter / union)
// Per-cluster pixel counts of a & b and a | b.  Each thread keeps one slot s for its whole
// run (its word stride is a multiple of S), so the 32 clusters of that slot are counted
// positionally in registers: 4-bit counters per bit (x >> r) & 0x11111111 for r = 0..3,
// spread into 8-bit counters every 12 words, and those added to the block's per-cluster
// counters every 252 words; the block's counters go to the global uint64 totals once.
__device__ __forceinline__ void iou_nib_flush(uint32_t* n, uint32_t* b) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        b[2 * r] += n[r] & 0x0F0F0F0Fu;
        b[2 * r + 1] += (n[r] >> 4) & 0x0F0F0F0Fu;
        n[r] = 0u;
    }
}

// byte k of b[2r + h] counts bit 8k + 4h + r
__device__ __forceinline__ void iou_byte_flush(uint32_t* b, unsigned int* hist, unsigned long long* glob, int base,
                                               int K) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int r = q >> 1, h = q & 1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t cnt = (b[q] >> (8 * k)) & 0xFFu;
            const int c = base + 8 * k + 4 * h + r;
            if (cnt && c < K) {
                if (hist) atomicAdd(hist + c, cnt);
                else atomicAdd(glob + c, (unsigned long long)cnt);
            }
        }
        b[q] = 0u;
    }
}

__global__ void __launch_bounds__(256) cluster_iou_kernel(int64_t npix, int S, int K, const int32_t* __restrict__ a,
                                                          const int32_t* __restrict__ b,
                                                          unsigned long long* __restrict__ inter,
                                                          unsigned long long* __restrict__ uni, int use_smem,
                                                          int64_t tstride) {
    extern __shared__ unsigned int hist[];  // inter[K] | union[K] when use_smem
    if (use_smem) {
        for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
    }
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nwords = npix * S;
    if (t < tstride) {
        const int base = (int)(t % S) * 32;
        uint32_t nI[4] = {0u, 0u, 0u, 0u}, nU[4] = {0u, 0u, 0u, 0u};
        uint32_t bI[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u}, bU[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        // four independent words per step (loads in flight); nibbles hold 12 words, bytes
        // 21 nibble flushes (252 words)
        int cn = 0, cb = 0;
        for (int64_t i = t; i < nwords; i += 4 * tstride) {
            uint32_t xs[4], ys[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t k = i + u * tstride;
                xs[u] = k < nwords ? (uint32_t)__ldcs(a + k) : 0u;
                ys[u] = k < nwords ? (uint32_t)__ldcs(b + k) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t ia = xs[u] & ys[u], ua = xs[u] | ys[u];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    nI[r] += (ia >> r) & 0x11111111u;
                    nU[r] += (ua >> r) & 0x11111111u;
                }
            }
            if (++cn == 3) {
                cn = 0;
                iou_nib_flush(nI, bI);
                iou_nib_flush(nU, bU);
                if (++cb == 21) {
                    cb = 0;
                    iou_byte_flush(bI, use_smem ? hist : nullptr, inter, base, K);
                    iou_byte_flush(bU, use_smem ? hist + K : nullptr, uni, base, K);
                }
            }
        }
        iou_nib_flush(nI, bI);
        iou_nib_flush(nU, bU);
        iou_byte_flush(bI, use_smem ? hist : nullptr, inter, base, K);
        iou_byte_flush(bU, use_smem ? hist + K : nullptr, uni, base, K);
    }
    if (use_smem) {
        __syncthreads();
        for (int c = threadIdx.x; c < K; c += blockDim.x) {
            if (hist[c]) atomicAdd(inter + c, (unsigned long long)hist[c]);
            if (hist[K + c]) atomicAdd(uni + c, (unsigned long long)hist[K + c]);
        }
    }
}

// ---- cluster planes ----------------------------------------------------------------------
// planes (B, 32 S, H, WQ) uint32, WQ = ceil(W / 32): bit (x & 31) of word x >> 5 of row y
// of plane c is bit c of pixel (y, x).  A CTA takes one image row, 256 pixels and 16 slots:
// the tile is read with whole 64-byte runs per pixel (16-byte loads), each thread turns one
// (32 pixels x 32 clusters) block around in registers, and the plane rows are written
// contiguously.  The input and output tiles share one shared-memory buffer (16.5 KB), so
// about 12 CTAs fit an SM and keep enough loads in flight: 0.109 ms per 256 MiB on GB300
// (4.9 TB/s); 512 x 8 tiles took 0.117 ms shared and 0.171 ms with separate buffers.
constexpr int kPlaneX = 256, kPlaneS = 16;
constexpr int kPlaneG = kPlaneX / 32;                   // pixel groups per tile
constexpr int kPlaneThreads = kPlaneG * kPlaneS;        // one thread per 32 x 32 block
constexpr int kTinRow = kPlaneS;                        // input tile: word (p, s) at
constexpr int kTinGrp = 32 * kTinRow + 4;               //   (p / 32) * kTinGrp + (p % 32) * kTinRow + s
constexpr int kToutRow = kPlaneG;                       // output tile: word (s, c, g) at
constexpr int kToutSlot = 32 * kToutRow + 8;            //   s * kToutSlot + c * kToutRow + g
constexpr int kPlaneIn = kPlaneG * kTinGrp, kPlaneOut = kPlaneS * kToutSlot;
constexpr int kPlaneV4 = kPlaneS / 4;                   // 16-byte loads per pixel
constexpr int kPlaneQ = kPlaneG / 4;                    // 16-byte stores per plane-row segment

// 32 x 32 bit transpose in registers: on return bit i of a[c] is bit c of the input a[i].
// Five stages swap the off-diagonal J x J blocks of every 2J x 2J block (J = 16 .. 1).
template <int J, uint32_t M>
__device__ __forceinline__ void transpose_stage(uint32_t (&a)[32]) {
#pragma unroll
    for (int k = 0; k < 32; k += 2 * J) {
#pragma unroll
        for (int i = 0; i < J; ++i) {
            const uint32_t t = ((a[k + i] >> J) ^ a[k + i + J]) & M;
            a[k + i + J] ^= t;
            a[k + i] ^= t << J;
        }
    }
}

__device__ __forceinline__ void transpose32_regs(uint32_t (&a)[32]) {
    transpose_stage<16, 0x0000FFFFu>(a);
    transpose_stage<8, 0x00FF00FFu>(a);
    transpose_stage<4, 0x0F0F0F0Fu>(a);
    transpose_stage<2, 0x33333333u>(a);
    transpose_stage<1, 0x55555555u>(a);
}

__global__ void __launch_bounds__(kPlaneThreads) bitset_to_planes_kernel(int B, int H, int W, int S,
                                                                        const int32_t* __restrict__ bitset,
                                                                        uint32_t* __restrict__ planes) {
    __shared__ __align__(16) uint32_t tbuf[kPlaneIn > kPlaneOut ? kPlaneIn : kPlaneOut];
    uint32_t* tin = tbuf;     // read into registers, then overwritten by the output tile
    uint32_t* tout = tbuf;
    const int WQ = (W + 31) >> 5;
    const int nxt = (W + kPlaneX - 1) / kPlaneX;
    const int xt = blockIdx.x % nxt, st = blockIdx.x / nxt;
    const int x0 = xt * kPlaneX, s0 = st * kPlaneS;
    const int y = blockIdx.y, b = blockIdx.z;
    const int64_t row = ((int64_t)b * H + y) * W;
    const int tid = threadIdx.x;
    if ((S & 3) == 0 && (((uintptr_t)bitset) & 15) == 0) {
        // 16-byte loads: pixel p's 16 slots are four int4 (S a multiple of 4)
#pragma unroll 4
        for (int i = tid; i < kPlaneX * kPlaneV4; i += kPlaneThreads) {
            const int p = i / kPlaneV4, h = i % kPlaneV4;
            const int x = x0 + p, sl = s0 + 4 * h;
            int4 v = make_int4(0, 0, 0, 0);
            if (x < W && sl < S) v = __ldg((const int4*)(bitset + (row + x) * S + sl));
            // 16-byte stores: a quarter warp writes two pixels' 16 words, all banks once
            *(int4*)(tin + (p >> 5) * kTinGrp + (p & 31) * kTinRow + 4 * h) = v;
        }
    } else {
        for (int i = tid; i < kPlaneX * kPlaneS; i += kPlaneThreads) {
            const int p = i / kPlaneS, sl = i - p * kPlaneS;
            const int x = x0 + p, sg = s0 + sl;
            tin[(p >> 5) * kTinGrp + (p & 31) * kTinRow + sl] =
                (x < W && sg < S) ? (uint32_t)__ldg(bitset + (row + x) * S + sg) : 0u;
        }
    }
    __syncthreads();
    {
        // thread (g, s): pixels 32 g .. 32 g + 31 of slot s; a warp holds g = 0..7 of four
        // slots (bank of input word i: 4 g + s + 16 i, of output word c: 8 s + g + 8 c,
        // distinct over the warp's threads for every i and c)
        const int g = tid % kPlaneG, sl = tid / kPlaneG;
        uint32_t a[32];
        const uint32_t* src = tin + g * kTinGrp + sl;
#pragma unroll
        for (int i = 0; i < 32; ++i) a[i] = src[i * kTinRow];
        __syncthreads();
        transpose32_regs(a);
        uint32_t* dst = tout + sl * kToutSlot + g;
#pragma unroll
        for (int c = 0; c < 32; ++c) dst[c * kToutRow] = a[c];
    }
    __syncthreads();
    const int Kp = 32 * S;
    const int q0 = x0 >> 5;
    const int nq = min(kPlaneG, WQ - q0);
    // one plane row segment (8 words) per (slot, cluster bit): 2 threads store 4 words each
    for (int i = tid; i < kPlaneS * 32 * kPlaneQ; i += kPlaneThreads) {
        const int quad = i % kPlaneQ, bit = (i / kPlaneQ) & 31, sl = i / (32 * kPlaneQ);
        const int sg = s0 + sl;
        if (sg >= S) continue;
        uint32_t* dst = planes + (((int64_t)b * Kp + 32 * sg + bit) * H + y) * WQ + q0;
        const uint32_t* src = tout + sl * kToutSlot + bit * kToutRow;
        const int g0 = 4 * quad;
        if (g0 + 4 <= nq && (((uintptr_t)(dst + g0)) & 15) == 0) {
            *(uint4*)(dst + g0) = *(const uint4*)(src + g0);   // 16-byte aligned: kToutSlot, kToutRow, g0 % 4 == 0
        } else {
            for (int gg = g0; gg < g0 + 4 && gg < nq; ++gg) dst[gg] = src[gg];
        }
    }
}

// Per-cluster counts from cluster planes: one CTA per (view, plane), popcounts of a & b
// and a | b over the plane's H * WQ contiguous words, one uint64 atomic per CTA and count.
__global__ void __launch_bounds__(256) planes_iou_kernel(int K, int Kp, int64_t words, const uint32_t* __restrict__ a,
                                                         const uint32_t* __restrict__ b,
                                                         unsigned long long* __restrict__ inter,
                                                         unsigned long long* __restrict__ uni) {
    const int c = blockIdx.x, v = blockIdx.y;
    if (c >= K) return;
    const int64_t off = ((int64_t)v * Kp + c) * words;
    const uint32_t* pa = a + off;
    const uint32_t* pb = b + off;
    unsigned int ni = 0, nu = 0;
    if ((words & 3) == 0 && ((((uintptr_t)pa) | ((uintptr_t)pb)) & 15) == 0) {
        const uint4* qa = (const uint4*)pa;
        const uint4* qb = (const uint4*)pb;
        for (int64_t i = threadIdx.x; i < words / 4; i += blockDim.x) {
            const uint4 x = __ldcs(qa + i), y = __ldcs(qb + i);
            ni += __popc(x.x & y.x) + __popc(x.y & y.y) + __popc(x.z & y.z) + __popc(x.w & y.w);
            nu += __popc(x.x | y.x) + __popc(x.y | y.y) + __popc(x.z | y.z) + __popc(x.w | y.w);
        }
    } else {
        for (int64_t i = threadIdx.x; i < words; i += blockDim.x) {
            const uint32_t x = pa[i], y = pb[i];
            ni += __popc(x & y);
            nu += __popc(x | y);
        }
    }
    for (int o = 16; o; o >>= 1) {
        ni += __shfl_xor_sync(0xffffffffu, ni, o);
        nu += __shfl_xor_sync(0xffffffffu, nu, o);
    }
    __shared__ unsigned int si[8], su[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        si[warp] = ni;
        su[warp] = nu;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ti = 0, tu = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            ti += si[w];
            tu += su[w];
        }
        if (ti) atomicAdd(inter + c, ti);
        if (tu) atomicAdd(uni + c, tu);
    }
}

// ---- plane rectangles ----------------------------------------------------------------
// A rectangle (y0, y1, q0, q1) per (view, plane): rows [y0, y1) x plane words [q0, q1),
// clamped to the plane; y0 >= y1 or q0 >= q1 is empty.
struct PlaneRect {
    int y0, y1, q0, q1;
    __device__ __forceinline__ bool empty() const { return y0 >= y1 || q0 >= q1; }
};

__device__ __forceinline__ PlaneRect plane_rect(const int4* __restrict__ rects, int64_t i, int H, int WQ) {
    const int4 r = __ldg(rects + i);
    PlaneRect p;
    p.y0 = max(r.x, 0);
    p.y1 = min(r.y, H);
    p.q0 = max(r.z, 0);
    p.q1 = min(r.w, WQ);
    return p;
}

// the words of a rectangle, one per thread in turn: row-major over (y0..y1) x (q0..q1)
template <class F>
__device__ __forceinline__ void for_rect_words(const PlaneRect& r, F f) {
    if (r.empty()) return;
    const int nq = r.q1 - r.q0;
    const int64_t n = (int64_t)(r.y1 - r.y0) * nq;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const int y = r.y0 + (int)(i / nq), q = r.q0 + (int)(i % nq);
        f(y, q);
    }
}

// zero each (view, plane)'s rectangle; one CTA per plane
__global__ void __launch_bounds__(256) planes_clear_rects_kernel(int Kp, int H, int WQ, uint32_t* __restrict__ planes,
                                                                 const int4* __restrict__ rects) {
    const int64_t pl = (int64_t)blockIdx.y * Kp + blockIdx.x;
    const PlaneRect r = plane_rect(rects, pl, H, WQ);
    uint32_t* p = planes + pl * H * WQ;
    for_rect_words(r, [&](int y, int q) { p[(int64_t)y * WQ + q] = 0u; });
}

// the smallest rectangle holding every non-zero word of each plane; one CTA per plane
__global__ void __launch_bounds__(256) planes_bounds_kernel(int Kp, int H, int WQ, const uint32_t* __restrict__ planes,
                                                            int4* __restrict__ rects) {
    const int64_t pl = (int64_t)blockIdx.y * Kp + blockIdx.x;
    __shared__ int b[4];
    if (threadIdx.x == 0) {
        b[0] = H;
        b[1] = 0;
        b[2] = WQ;
        b[3] = 0;
    }
    __syncthreads();
    const uint32_t* p = planes + pl * H * WQ;
    const int64_t n = (int64_t)H * WQ;
    int y0 = H, y1 = 0, q0 = WQ, q1 = 0;
    auto take = [&](int64_t i) {
        const int y = (int)(i / WQ), q = (int)(i % WQ);
        y0 = min(y0, y);
        y1 = max(y1, y + 1);
        q0 = min(q0, q);
        q1 = max(q1, q + 1);
    };
    if ((n & 3) == 0 && ((uintptr_t)p & 15) == 0) {
        // 16-byte loads; a plane is mostly zero words, so most quads are skipped whole
        const uint4* p4 = (const uint4*)p;
        for (int64_t i = threadIdx.x; i < (n >> 2); i += blockDim.x) {
            const uint4 v = __ldcs(p4 + i);
            if ((v.x | v.y | v.z | v.w) == 0u) continue;
            if (v.x) take(4 * i);
            if (v.y) take(4 * i + 1);
            if (v.z) take(4 * i + 2);
            if (v.w) take(4 * i + 3);
        }
    } else {
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            if (__ldcs(p + i) != 0u) take(i);
    }
    if (y1 > 0) {
        atomicMin(b + 0, y0);
        atomicMax(b + 1, y1);
        atomicMin(b + 2, q0);
        atomicMax(b + 3, q1);
    }
    __syncthreads();
    if (threadIdx.x == 0) rects[pl] = make_int4(b[0], b[1], b[2], b[3]);
}

// Per-cluster counts over the bounding rectangle of both planes' rectangles (every set bit
// of either plane lies inside its rectangle); *xor_total += sum over all planes of
// popc(a ^ b) = union - inter.
__global__ void __launch_bounds__(256) planes_iou_rects_kernel(int K, int Kp, int H, int WQ,
                                                               const uint32_t* __restrict__ a,
                                                               const uint32_t* __restrict__ b,
                                                               const int4* __restrict__ ra,
                                                               const int4* __restrict__ rb,
                                                               unsigned long long* __restrict__ inter,
                                                               unsigned long long* __restrict__ uni,
                                                               unsigned long long* __restrict__ xor_total) {
    const int c = blockIdx.x;
    const int64_t pl = (int64_t)blockIdx.y * Kp + c;
    const PlaneRect x = plane_rect(ra, pl, H, WQ), y = plane_rect(rb, pl, H, WQ);
    PlaneRect r;
    if (x.empty()) r = y;
    else if (y.empty()) r = x;
    else {
        r.y0 = min(x.y0, y.y0);
        r.y1 = max(x.y1, y.y1);
        r.q0 = min(x.q0, y.q0);
        r.q1 = max(x.q1, y.q1);
    }
    const uint32_t* pa = a + pl * H * WQ;
    const uint32_t* pb = b + pl * H * WQ;
    unsigned int ni = 0, nu = 0;
    for_rect_words(r, [&](int yy, int q) {
        const int64_t i = (int64_t)yy * WQ + q;
        const uint32_t u = pa[i], v = pb[i];
        ni += __popc(u & v);
        nu += __popc(u | v);
    });
    for (int o = 16; o; o >>= 1) {
        ni += __shfl_xor_sync(0xffffffffu, ni, o);
        nu += __shfl_xor_sync(0xffffffffu, nu, o);
    }
    __shared__ unsigned int si[8], su[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        si[warp] = ni;
        su[warp] = nu;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ti = 0, tu = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            ti += si[w];
            tu += su[w];
        }
        if (c < K) {
            if (ti) atomicAdd(inter + c, ti);
            if (tu) atomicAdd(uni + c, tu);
        }
        if (xor_total && tu > ti) atomicAdd(xor_total, tu - ti);
    }
}

}  // namespace s2c

using namespace s2c;

extern "C" s2c_status s2c_xor_popcount(int64_t nwords, const int32_t* a, const int32_t* b, uint64_t* total,
                                       s2c_stream stream) {
    S2C_REQUIRE(nwords >= 0 && total, "xor_popcount: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(total, 0, sizeof(uint64_t), st);
    if (e != cudaSuccess) return cuda_status(e, "xor_popcount: memset");
    if (nwords == 0) return S2C_OK;
    S2C_REQUIRE(a && b && ((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0, "xor_popcount: bitsets must be 16-byte aligned");
    const unsigned grid = (unsigned)std::min<int64_t>((nwords / 4 + 255) / 256 + 1, (int64_t)num_sms() * 8);
    xor_popcount_kernel<<<grid, 256, 0, st>>>(nwords, a, b, (unsigned long long*)total);
    S2C_CHECK_LAUNCH("xor_popcount_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_cluster_iou_counts(int64_t npix, int S, int K, const int32_t* a, const int32_t* b,
                                             uint64_t* inter, uint64_t* uni, s2c_stream stream) {
    S2C_REQUIRE(npix >= 0 && S > 0 && K >= 0 && K <= 32 * S, "cluster_iou_counts: bad sizes");
    S2C_REQUIRE(inter && uni, "cluster_iou_counts: null output");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(inter, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(uni, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e != cudaSuccess) return cuda_status(e, "cluster_iou_counts: memset");
    if (npix == 0 || K == 0) return S2C_OK;
    S2C_REQUIRE(a && b, "cluster_iou_counts: null input");
    const size_t smem = (size_t)2 * K * sizeof(unsigned int);
    const int use_smem = smem <= 48 * 1024;
    int64_t grid = std::min<int64_t>((npix * S + 255) / 256, (int64_t)num_sms() * 8);
    grid = std::max<int64_t>(grid, (S + 255) / 256);
    // every thread's stride is a whole number of pixels, so its slot never changes
    const int64_t tstride = (grid * 256 / S) * S;
    cluster_iou_kernel<<<(unsigned)grid, 256, use_smem ? smem : 0, st>>>(
        npix, S, K, a, b, (unsigned long long*)inter, (unsigned long long*)uni, use_smem, tstride);
    S2C_CHECK_LAUNCH("cluster_iou_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_popcount_bitset(int64_t npix, int S, const int32_t* bitset, float* count_image,
                                          s2c_stream stream) {
    S2C_REQUIRE(npix >= 0 && S > 0, "popcount_bitset: bad sizes");
    if (npix == 0) return S2C_OK;
    S2C_REQUIRE(bitset && count_image, "popcount_bitset: null pointer");
    S2C_REQUIRE((S & 3) != 0 || ((uintptr_t)bitset & 15) == 0, "popcount_bitset: bitset must be 16-byte aligned");
    S2C_REQUIRE((npix + kBitsPix - 1) / kBitsPix < (1LL << 31), "popcount_bitset: too many pixels");
    popcount_kernel<<<(unsigned)((npix + kBitsPix - 1) / kBitsPix), kBitsPix, 0, (cudaStream_t)stream>>>(
        npix, S, bitset, count_image);
    S2C_CHECK_LAUNCH("popcount_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_accumulate_bitset_rgb(int64_t npix, int S, const int32_t* bitset, int K, const float* rgb,
                                                float* accum, s2c_stream stream) {
    S2C_REQUIRE(npix >= 0 && S > 0 && K >= 0, "accumulate_bitset_rgb: bad sizes");
    S2C_REQUIRE(S * 32 >= K, "Too few slots for the number of clusters.");
    if (npix == 0) return S2C_OK;
    S2C_REQUIRE(bitset && accum && (K == 0 || rgb), "accumulate_bitset_rgb: null pointer");
    S2C_REQUIRE((npix + kBitsPix - 1) / kBitsPix < (1LL << 31), "accumulate_bitset_rgb: too many pixels");
    accumulate_rgb_kernel<<<(unsigned)((npix + kBitsPix - 1) / kBitsPix), kBitsPix, 0, (cudaStream_t)stream>>>(
        npix, S, bitset, K, rgb, accum);
    S2C_CHECK_LAUNCH("accumulate_rgb_kernel");
    return S2C_OK;
}

extern "C" size_t s2c_bitset_planes_size(int B, int H, int W, int S) {
    if (B <= 0 || H <= 0 || W <= 0 || S <= 0) return 0;
    return (size_t)B * 32 * S * H * ((W + 31) / 32) * sizeof(uint32_t);
}

extern "C" s2c_status s2c_bitset_to_planes(int B, int H, int W, int S, const int32_t* bitset, uint32_t* planes,
                                           s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && S > 0 && H <= 65535 && B <= 65535, "bitset_to_planes: bad sizes");
    if (B == 0 || H == 0 || W == 0) return S2C_OK;
    S2C_REQUIRE(bitset && planes, "bitset_to_planes: null pointer");
    const int nxt = (W + kPlaneX - 1) / kPlaneX, nst = (S + kPlaneS - 1) / kPlaneS;
    S2C_REQUIRE((int64_t)nxt * nst < (1LL << 31), "bitset_to_planes: too many tiles");
    dim3 grid((unsigned)(nxt * nst), (unsigned)H, (unsigned)B);
    bitset_to_planes_kernel<<<grid, kPlaneThreads, 0, (cudaStream_t)stream>>>(B, H, W, S, bitset, planes);
    S2C_CHECK_LAUNCH("bitset_to_planes_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_cluster_iou_counts_planes(int B, int H, int W, int S, int K, const uint32_t* a,
                                                    const uint32_t* b, uint64_t* inter, uint64_t* uni,
                                                    s2c_stream stream) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && S > 0 && K >= 0 && K <= 32 * S && B <= 65535,
                "cluster_iou_counts_planes: bad sizes");
    S2C_REQUIRE(inter && uni, "cluster_iou_counts_planes: null output");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(inter, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(uni, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e != cudaSuccess) return cuda_status(e, "cluster_iou_counts_planes: memset");
    if (B == 0 || H == 0 || W == 0 || K == 0) return S2C_OK;
    S2C_REQUIRE(a && b, "cluster_iou_counts_planes: null input");
    const int64_t words = (int64_t)H * ((W + 31) / 32);
    planes_iou_kernel<<<dim3((unsigned)K, (unsigned)B), 256, 0, st>>>(K, 32 * S, words, a, b,
                                                                        (unsigned long long*)inter,
                                                                        (unsigned long long*)uni);
    S2C_CHECK_LAUNCH("planes_iou_kernel");
    return S2C_OK;
}

static s2c_status check_rects(const char* what, int B, int H, int W, int S, const void* planes, const void* rects) {
    S2C_REQUIRE(B >= 0 && H >= 0 && W >= 0 && S > 0 && B <= 65535 && 32LL * S <= 2147483647LL, "%s: bad sizes", what);
    S2C_REQUIRE(planes && rects, "%s: null pointer", what);
    S2C_REQUIRE(((uintptr_t)rects & 15) == 0, "%s: rects must be 16-byte aligned", what);
    return S2C_OK;
}

extern "C" s2c_status s2c_planes_clear_rects(int B, int H, int W, int S, uint32_t* planes, const int32_t* rects,
                                             s2c_stream stream) {
    if (B == 0 || H == 0 || W == 0) return S2C_OK;
    s2c_status st = check_rects("planes_clear_rects", B, H, W, S, planes, rects);
    if (st != S2C_OK) return st;
    planes_clear_rects_kernel<<<dim3((unsigned)(32 * S), (unsigned)B), 256, 0, (cudaStream_t)stream>>>(
        32 * S, H, (W + 31) / 32, planes, (const int4*)rects);
    S2C_CHECK_LAUNCH("planes_clear_rects_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_planes_bounds(int B, int H, int W, int S, const uint32_t* planes, int32_t* rects,
                                        s2c_stream stream) {
    if (B == 0 || H == 0 || W == 0) return S2C_OK;
    s2c_status st = check_rects("planes_bounds", B, H, W, S, planes, rects);
    if (st != S2C_OK) return st;
    planes_bounds_kernel<<<dim3((unsigned)(32 * S), (unsigned)B), 256, 0, (cudaStream_t)stream>>>(
        32 * S, H, (W + 31) / 32, planes, (int4*)rects);
    S2C_CHECK_LAUNCH("planes_bounds_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_cluster_iou_counts_planes_rects(int B, int H, int W, int S, int K, const uint32_t* a,
                                                          const uint32_t* b, const int32_t* rects_a,
                                                          const int32_t* rects_b, uint64_t* inter, uint64_t* uni,
                                                          uint64_t* xor_total, s2c_stream stream) {
    S2C_REQUIRE(K >= 0 && K <= 32 * S, "cluster_iou_counts_planes_rects: bad K");
    S2C_REQUIRE(inter && uni, "cluster_iou_counts_planes_rects: null output");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(inter, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(uni, 0, sizeof(uint64_t) * (size_t)K, st);
    if (e == cudaSuccess && xor_total) e = cudaMemsetAsync(xor_total, 0, sizeof(uint64_t), st);
    if (e != cudaSuccess) return cuda_status(e, "cluster_iou_counts_planes_rects: memset");
    if (B == 0 || H == 0 || W == 0) return S2C_OK;
    s2c_status s1 = check_rects("cluster_iou_counts_planes_rects", B, H, W, S, a, rects_a);
    if (s1 == S2C_OK) s1 = check_rects("cluster_iou_counts_planes_rects", B, H, W, S, b, rects_b);
    if (s1 != S2C_OK) return s1;
    planes_iou_rects_kernel<<<dim3((unsigned)(32 * S), (unsigned)B), 256, 0, st>>>(
        K, 32 * S, H, (W + 31) / 32, a, b, (const int4*)rects_a, (const int4*)rects_b, (unsigned long long*)inter,
        (unsigned long long*)uni, (unsigned long long*)xor_total);
    S2C_CHECK_LAUNCH("planes_iou_rects_kernel");
    return S2C_OK;
}
