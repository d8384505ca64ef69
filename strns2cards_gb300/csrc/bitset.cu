// Per-pixel bitset reductions (the reference's bitset_utils.cu) and bitset comparisons.
#include "common.cuh"

namespace s2c {

// bitset_utils.cu:37-52; one thread per pixel, 16-byte loads when S % 4 == 0
__global__ void __launch_bounds__(256) popcount_kernel(int64_t npix, int S, const int32_t* __restrict__ bits,
                                                       float* __restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int32_t* row = bits + p * S;
    int n = 0;
    if ((S & 3) == 0) {
        const int4* r4 = reinterpret_cast<const int4*>(row);
        for (int s = 0; s < (S >> 2); ++s) {
            const int4 v = __ldg(r4 + s);
            n += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        }
    } else {
        for (int s = 0; s < S; ++s) n += __popc(__ldg(row + s));
    }
    out[p] = (float)n;
}

// bitset_utils.cu:6-35: clusters are visited in increasing id order, the same float
// summation order as the reference, so the sums are bit-identical.
__global__ void __launch_bounds__(256) accumulate_rgb_kernel(int64_t npix, int S, const int32_t* __restrict__ bits,
                                                             int K, const float* __restrict__ rgb,
                                                             float* __restrict__ out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float r = 0.f, g = 0.f, b = 0.f;
    for (int s = 0; s < S; ++s) {
        uint32_t m = (uint32_t)__ldg(bits + p * S + s);
        while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            const int c = s * 32 + j;
            if (c >= K) continue;
            r = __fadd_rn(r, __ldg(rgb + 3 * c));
            g = __fadd_rn(g, __ldg(rgb + 3 * c + 1));
            b = __fadd_rn(b, __ldg(rgb + 3 * c + 2));
        }
    }
    out[3 * p] = r;
    out[3 * p + 1] = g;
    out[3 * p + 2] = b;
}

}  // namespace s2c

using namespace s2c;

extern "C" s2c_status s2c_popcount_bitset(int64_t npix, int S, const int32_t* bitset, float* count_image,
                                          s2c_stream stream) {
    S2C_REQUIRE(npix >= 0 && S > 0, "popcount_bitset: bad sizes");
    if (npix == 0) return S2C_OK;
    S2C_REQUIRE(bitset && count_image, "popcount_bitset: null pointer");
    S2C_REQUIRE((S & 3) != 0 || ((uintptr_t)bitset & 15) == 0, "popcount_bitset: bitset must be 16-byte aligned");
    popcount_kernel<<<grid_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(npix, S, bitset, count_image);
    S2C_CHECK_LAUNCH("popcount_kernel");
    return S2C_OK;
}

extern "C" s2c_status s2c_accumulate_bitset_rgb(int64_t npix, int S, const int32_t* bitset, int K, const float* rgb,
                                                float* accum, s2c_stream stream) {
    S2C_REQUIRE(npix >= 0 && S > 0 && K >= 0, "accumulate_bitset_rgb: bad sizes");
    S2C_REQUIRE(S * 32 >= K, "Too few slots for the number of clusters.");
    if (npix == 0) return S2C_OK;
    S2C_REQUIRE(bitset && accum && (K == 0 || rgb), "accumulate_bitset_rgb: null pointer");
    accumulate_rgb_kernel<<<grid_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(npix, S, bitset, K, rgb, accum);
    S2C_CHECK_LAUNCH("accumulate_rgb_kernel");
    return S2C_OK;
}
