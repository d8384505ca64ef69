// Compacted fragment lists in two passes over a raw index space, without the raw list.
//
// The reference lists one raw fragment per unit of work -- every bounding-box pixel of a
// triangle, every DDA step of a segment -- marks the rejected ones (-1) and compacts the list
// in order.  Here pass 1 evaluates every raw index and sets one bit per accepted fragment, a
// scan of the bit words' popcounts places each accepted fragment, and pass 2 evaluates the
// accepted indices again and writes them at their places: the same list, without writing,
// clearing and re-reading the raw one.
//
// The raw index space is the inclusive prefix of the owners' counts (int32, owners
// 0 .. n - 1).  Warps take kListChunk-index chunks and keep a window of 32 consecutive
// owners' prefix values in their lanes; each lane finds the owner of its index by a 5-step
// shuffle search instead of a binary search over the whole prefix.
#pragma once
#include <algorithm>

#include "common.cuh"

namespace s2c {

constexpr int kListChunk = 1024;   // a multiple of 32: a mask word never straddles two chunks

// pass 1 (kWrite = false): eval(owner, k) -> accepted, setting bits of mask (zeroed before);
// pass 2: for the accepted indices, write(owner, k, place).  eval / write are device lambdas.
template <bool kWrite, class Eval, class Write>
__device__ __forceinline__ void list_pass(int64_t n, uint32_t F, const int32_t* __restrict__ prefix,
                                          uint32_t* __restrict__ mask, const int32_t* __restrict__ wpre, Eval eval,
                                          Write write) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nch = ((int64_t)F + kListChunk - 1) / kListChunk;
    for (int64_t ch = warp0; ch < nch; ch += nwarps) {
        const uint32_t c0 = (uint32_t)(ch * kListChunk);
        const uint32_t c1 = (uint32_t)min((int64_t)F, (ch + 1) * kListChunk);
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if ((uint32_t)__ldg(prefix + mid) <= c0) lo = mid + 1;
            else hi = mid;
        }
        int64_t t0 = lo;
        uint32_t start = t0 > 0 ? (uint32_t)__ldg(prefix + t0 - 1) : 0u;
        uint32_t pre = t0 + lane < n ? (uint32_t)__ldg(prefix + t0 + lane) : 0xffffffffu;
        uint32_t base = c0;
        while (base < c1) {
            for (;;) {
                const unsigned m = __ballot_sync(0xffffffffu, pre <= base);
                if (!m) break;
                const int adv = __popc(m);
                start = __shfl_sync(0xffffffffu, pre, adv - 1);
                t0 += adv;
                pre = t0 + lane < n ? (uint32_t)__ldg(prefix + t0 + lane) : 0xffffffffu;
            }
            const uint32_t wend = __shfl_sync(0xffffffffu, pre, 31);
            const uint32_t end = min(min(c1, base + 32u), wend);
            const uint32_t j = base + lane;
            int ow = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1) {
                const uint32_t pv = __shfl_sync(0xffffffffu, pre, ow + step - 1);
                if (pv <= j) ow += step;
            }
            const uint32_t prev = __shfl_sync(0xffffffffu, pre, ow > 0 ? ow - 1 : 0);
            // the owner of j < end has index t0 + ow < n (its prefix exceeds j)
            const int64_t o = t0 + ow;
            const int k = (int)(j - (ow > 0 ? prev : start));
            if (!kWrite) {
                const bool acc = j < end && eval(o, k);
                // lanes 0 .. end - base - 1 hold indices base .. end - 1
                const unsigned m = __ballot_sync(0xffffffffu, acc);
                if (lane == 0 && m) {
                    const uint32_t w = base >> 5, sh = base & 31;
                    atomicOr(mask + w, m << sh);
                    if (sh && (m >> (32 - sh))) atomicOr(mask + w + 1, m >> (32 - sh));
                }
            } else if (j < end) {
                const uint32_t w = j >> 5, word = mask[w];
                if ((word >> (j & 31)) & 1u) {
                    const int64_t at = (int64_t)(w ? (uint32_t)wpre[w - 1] : 0u) + __popc(word & ((1u << (j & 31)) - 1u));
                    write(o, k, at);
                }
            }
            base = end;
        }
    }
}

// Workspace of a two-pass list over F raw indices: the mask, its words' inclusive prefix,
// the total and the scan's scratch.
struct ListWs {
    uint32_t* mask;
    int32_t* wpre;
    int64_t* total;
    void* scan;
};

size_t list_carve(int64_t F, void* base, size_t cap, ListWs* w);

// after pass 1: the words' popcounts, their inclusive prefix and the accepted count (host;
// synchronises the stream)
s2c_status list_count(int64_t F, const ListWs& w, int64_t* num, cudaStream_t st);

inline unsigned list_grid(int64_t F) {
    return (unsigned)std::min<int64_t>((F + kListChunk - 1) / kListChunk / 8 + 1, (int64_t)num_sms() * 8);
}

}  // namespace s2c
