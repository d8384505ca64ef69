// Strand curve operators: arclength, Gaussian-in-arclength smoothing, arclength skinning.
//
// Reference: curve_utils.cu:24-68 (smooth_strands_kernel) and :70-131 (skinning_kernel), one
// thread per strand walking all V x V point pairs straight from global memory with a
// 12-byte stride per thread.  Here a CTA takes a group of whole strands, stages their
// points (and handles / rotations for skinning) in shared memory with coalesced loads,
// computes the arclength in the CTA when the caller passes none (a warp scan per strand),
// and gives every point its own thread, so the O(V^2) pair loop reads broadcast shared
// memory.  Per point i the sum runs over j = 0..V-1 in order and skips pairs with
// |a_i - a_j| > 3 beta exactly as the reference does; weights exp(-d^2 / beta^2) use expf.
// With the arclength computed in the kernel the loop visits only the run of j inside the
// cutoff (same terms, same order).
#include <algorithm>

#include "common.cuh"
#include "scan.cuh"
#include "strand_sums.cuh"

namespace s2c {
namespace {

constexpr int kCurveThreads = 256;
constexpr int kCurveSmem = 48 * 1024;           // bytes of staged strand data per CTA
constexpr int kSmoothBytes = 16;                // x(3) + arclength
constexpr int kSkinBytes = 76;                  // x(3) + arclength + h(3) + c(3) + R(9)
constexpr int kMaxArcOnly = kCurveSmem / 4;     // longest strand whose arclength fits alone

struct CurveArgs {
    int N, V, spb, ngroups;
    bool staged;                                // whole group staged (else only arclength)
    const float* x;
    const float* arc;                           // nullable: computed in the kernel
    const float* h;
    const float* c;
    const float* R;
    float* out;
    float beta;
};

template <bool kSkin>
__global__ void __launch_bounds__(kCurveThreads) curve_kernel(CurveArgs a) {
    extern __shared__ __align__(16) float sm[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int V = a.V;
    const int cap = a.spb * V;
    // shared layout (staged): x[3 cap] | arc[cap] | h[3 cap] | c[3 cap] | R[9 cap]
    float* sx = sm;
    float* sarc = a.staged ? sm + 3 * cap : sm;
    float* sh = sm + 4 * cap;
    float* sc = sm + 7 * cap;
    float* sR = sm + 10 * cap;
    const float inv_beta2 = __fdiv_rn(1.0f, __fmul_rn(a.beta, a.beta));
    const float cutoff = __fmul_rn(3.0f, a.beta);

    for (int g = blockIdx.x; g < a.ngroups; g += gridDim.x) {
        const int64_t s0 = (int64_t)g * a.spb;
        const int ns = (int)(a.N - s0 < a.spb ? a.N - s0 : a.spb);
        const int P = ns * V;
        const int64_t p0 = s0 * V;
        const float* gx = a.x + 3 * p0;
        if (a.staged) {
            for (int k = tid; k < 3 * P; k += kCurveThreads) sx[k] = __ldg(gx + k);
            if (kSkin) {
                for (int k = tid; k < 3 * P; k += kCurveThreads) {
                    sh[k] = __ldg(a.h + 3 * p0 + k);
                    sc[k] = __ldg(a.c + 3 * p0 + k);
                }
                for (int k = tid; k < 9 * P; k += kCurveThreads) sR[k] = __ldg(a.R + 9 * p0 + k);
            }
        }
        if (a.arc) {
            for (int k = tid; k < P; k += kCurveThreads) sarc[k] = __ldg(a.arc + p0 + k);
            __syncthreads();
        } else {
            __syncthreads();
            const float* xs = a.staged ? sx : gx;
            for (int s = warp; s < ns; s += kCurveThreads / 32) warp_arclength(xs + 3 * s * V, V, sarc + s * V, lane);
            __syncthreads();
        }
        const float* X = a.staged ? sx : gx;
        const float* Hh = a.staged ? sh : a.h + 3 * p0;
        const float* Cc = a.staged ? sc : a.c + 3 * p0;
        const float* RR = a.staged ? sR : a.R + 9 * p0;
        for (int p = tid; p < P; p += kCurveThreads) {
            const int sl = p / V;
            const int i = p - sl * V;
            const int b = sl * V;
            float o3[3];
            if (kSkin)
                skin_point(X + 3 * b, sarc + b, Hh + 3 * b, Cc + 3 * b, RR + 9 * b, V, i, cutoff, inv_beta2, !a.arc, o3);
            else
                smooth_point(X + 3 * b, sarc + b, V, i, cutoff, inv_beta2, !a.arc, o3);
            float* o = a.out + 3 * (p0 + p);
            o[0] = o3[0];
            o[1] = o3[1];
            o[2] = o3[2];
        }
        __syncthreads();
    }
}

__global__ void arclength_kernel(int N, int V, const float* __restrict__ x, float* __restrict__ arc) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = w0; s < N; s += nw) warp_arclength(x + 3 * s * V, V, arc + s * V, lane);
}

s2c_status launch_curves(bool skin, int N, int V, const float* x, const float* arc, const float* h,
                         const float* c, const float* R, float* out, float beta, cudaStream_t st) {
    const char* name = skin ? "skinning" : "smooth_strands";
    S2C_REQUIRE(N >= 0 && V >= 0, "%s: negative size (N=%d, V=%d)", name, N, V);
    S2C_REQUIRE(N == 0 || V == 0 || (x && out), "%s: null strands or output", name);
    S2C_REQUIRE(!skin || N == 0 || V == 0 || (h && c && R), "%s: null handle, canonical or rotation array", name);
    if (N == 0 || V == 0) return S2C_OK;
    const int bpp = skin ? kSkinBytes : kSmoothBytes;
    CurveArgs a{};
    a.N = N; a.V = V; a.x = x; a.arc = arc; a.h = h; a.c = c; a.R = R; a.out = out; a.beta = beta;
    const int fit = kCurveSmem / bpp / V;       // whole strands a CTA can stage
    size_t smem;
    if (fit >= 1) {
        // enough strands per CTA to fill its threads, few enough to give every SM work
        const int want_threads = (kCurveThreads + V - 1) / V;
        const int want_spread = (int)std::max<int64_t>(1, ((int64_t)N + 4 * num_sms() - 1) / (4 * num_sms()));
        a.spb = std::min(fit, std::max(want_threads, std::min(want_spread, fit)));
        a.staged = true;
        smem = (size_t)a.spb * V * bpp;
    } else {
        S2C_REQUIRE(V <= kMaxArcOnly, "%s: strands of %d points exceed the staged limit of %d", name, V, kMaxArcOnly);
        a.spb = 1;
        a.staged = false;
        smem = (size_t)V * 4;
    }
    a.ngroups = (int)(((int64_t)N + a.spb - 1) / a.spb);
    const int blocks = (int)std::min<int64_t>(a.ngroups, (int64_t)num_sms() * 8);
    if (skin)
        curve_kernel<true><<<blocks, kCurveThreads, smem, st>>>(a);
    else
        curve_kernel<false><<<blocks, kCurveThreads, smem, st>>>(a);
    S2C_CHECK_LAUNCH(name);
    return S2C_OK;
}

// Arclength resampling of ragged strands (the reference's host resample_strands_by_arclength,
// hair_loader.cpp:261-307) with the same FP32 operations in the same order per strand:
// bit-identical to the host version.  ends = inclusive prefix of the point counts.
// The same per strand with a warp: the strand's points are read into shared memory with
// coalesced loads, the lanes take the segment lengths, one lane runs the cumulative sum in
// order (the host's summation order, so the arclengths are bit-identical), the lanes
// normalise and take the output samples.  Strands longer than kResampleCap points go to
// resample_kernel (its thread per strand works from global memory).
constexpr int kResampleCap = 384, kResampleWarps = 4;

__global__ void __launch_bounds__(32 * kResampleWarps) resample_warp_kernel(
    int ns, const int32_t* __restrict__ counts, const int32_t* __restrict__ ends, const float* __restrict__ pts,
    int64_t npts, int T, float* __restrict__ out, int32_t* __restrict__ long_list, int32_t* __restrict__ n_long,
    int32_t* __restrict__ bad) {
    __shared__ float s_p[kResampleWarps][3 * kResampleCap];
    __shared__ float s_L[kResampleWarps][kResampleCap];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float* P = s_p[w];
    float* L = s_L[w];
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < ns; i += nw) {
        const int N = counts[i];
        const int64_t at = (int64_t)ends[i] - N;
        float* o = out + (int64_t)i * T * 3;
        if (N < 2 || at < 0 || at + N > npts) {   // too short, or counts overrunning the points
            if (lane == 0) atomicMax(bad, 1);
            for (int k = lane; k < 3 * T; k += 32) o[k] = __int_as_float(0x7fc00000);
            continue;
        }
        if (N > kResampleCap) {
            if (lane == 0) long_list[atomicAdd(n_long, 1)] = i;
            continue;
        }
        const float* p = pts + 3 * at;
        for (int k = lane; k < 3 * N; k += 32) P[k] = __ldg(p + k);
        __syncwarp();
        for (int j = 1 + lane; j < N; j += 32) {
            const float dx = __fsub_rn(P[3 * j], P[3 * j - 3]);
            const float dy = __fsub_rn(P[3 * j + 1], P[3 * j - 2]);
            const float dz = __fsub_rn(P[3 * j + 2], P[3 * j - 1]);
            L[j] = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
        }
        __syncwarp();
        if (lane == 0) {
            float acc = 0.f;
            L[0] = 0.f;
            for (int j = 1; j < N; ++j) {
                acc = __fadd_rn(acc, L[j]);
                L[j] = acc;
            }
        }
        __syncwarp();
        const float total = L[N - 1];
        __syncwarp();
        for (int j = lane; j < N; j += 32) L[j] = __fdiv_rn(L[j], total);
        __syncwarp();
        for (int j = lane; j + 1 < T; j += 32) {
            const float t = __fdiv_rn((float)j, (float)(T - 1));
            int lo = 0, hi = N;   // first index with L > t
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (!(t < L[mid])) lo = mid + 1;
                else hi = mid;
            }
            const int k = min(max(lo, 1), N - 1);
            const float den = __fsub_rn(L[k], L[k - 1]);
            const float t0 = __fdiv_rn(__fsub_rn(L[k], t), den);
            const float t1 = __fdiv_rn(__fsub_rn(t, L[k - 1]), den);
#pragma unroll
            for (int c = 0; c < 3; ++c)
                o[3 * j + c] = __fadd_rn(__fmul_rn(t0, P[3 * (k - 1) + c]), __fmul_rn(t1, P[3 * k + c]));
        }
        if (lane < 3) o[3 * (T - 1) + lane] = P[3 * (N - 1) + lane];
        __syncwarp();
    }
}

// the strands resample_warp_kernel left (longer than kResampleCap points): a thread each
__global__ void resample_long_kernel(const int32_t* __restrict__ long_list, const int32_t* __restrict__ n_long,
                                     const int32_t* __restrict__ counts, const int32_t* __restrict__ ends,
                                     const float* __restrict__ pts, int64_t npts, int T, float* __restrict__ len,
                                     float* __restrict__ out) {
    const int n = *n_long;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int i = long_list[q];
        const int N = counts[i];
        const int64_t at = (int64_t)ends[i] - N;
        float* o = out + (int64_t)i * T * 3;
        const float* p = pts + 3 * at;
        float* L = len + at;
        L[0] = 0.f;
        for (int j = 1; j < N; ++j) {
            const float dx = __fsub_rn(p[3 * j], p[3 * j - 3]);
            const float dy = __fsub_rn(p[3 * j + 1], p[3 * j - 2]);
            const float dz = __fsub_rn(p[3 * j + 2], p[3 * j - 1]);
            L[j] = __fadd_rn(L[j - 1], __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                           __fmul_rn(dz, dz))));
        }
        const float total = L[N - 1];
        for (int j = 0; j < N; ++j) L[j] = __fdiv_rn(L[j], total);
        for (int j = 0; j + 1 < T; ++j) {
            const float t = __fdiv_rn((float)j, (float)(T - 1));
            int lo = 0, hi = N;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (!(t < L[mid])) lo = mid + 1;
                else hi = mid;
            }
            const int k = min(max(lo, 1), N - 1);
            const float den = __fsub_rn(L[k], L[k - 1]);
            const float t0 = __fdiv_rn(__fsub_rn(L[k], t), den);
            const float t1 = __fdiv_rn(__fsub_rn(t, L[k - 1]), den);
#pragma unroll
            for (int c = 0; c < 3; ++c)
                o[3 * j + c] = __fadd_rn(__fmul_rn(t0, p[3 * (k - 1) + c]), __fmul_rn(t1, p[3 * k + c]));
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) o[3 * (T - 1) + c] = p[3 * (N - 1) + c];
    }
}

}  // namespace
}  // namespace s2c

extern "C" {

S2C_API s2c_status s2c_compute_arclength(int N, int V, const float* strands, float* arclength,
                                         s2c_stream stream) {
    S2C_REQUIRE(N >= 0 && V >= 0, "compute_arclength: negative size (N=%d, V=%d)", N, V);
    if (N == 0 || V == 0) return S2C_OK;
    S2C_REQUIRE(strands && arclength, "compute_arclength: null pointer");
    const int threads = 256;
    const unsigned blocks = s2c::grid_for((int64_t)N * 32, threads, (int64_t)s2c::num_sms() * 16);
    s2c::arclength_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(N, V, strands, arclength);
    S2C_CHECK_LAUNCH("compute_arclength");
    return S2C_OK;
}

S2C_API s2c_status s2c_smooth_strands(int N, int V, const float* strands, const float* arclength,
                                      float* smoothed_strands, float beta, s2c_stream stream) {
    return s2c::launch_curves(false, N, V, strands, arclength, nullptr, nullptr, nullptr, smoothed_strands,
                              beta, (cudaStream_t)stream);
}

S2C_API s2c_status s2c_skinning(int N, int V, const float* strands, const float* arclength,
                                const float* handle_strands, const float* canonical_handles,
                                const float* R, float* skinned_strands, float beta, s2c_stream stream) {
    return s2c::launch_curves(true, N, V, strands, arclength, handle_strands, canonical_handles, R,
                              skinned_strands, beta, (cudaStream_t)stream);
}

}  // extern "C"

extern "C" size_t s2c_resample_strands_workspace_size(int num_strands, int64_t num_points) {
    const size_t ns = (size_t)(num_strands > 0 ? num_strands : 1);
    return 2 * s2c::align_up(ns * 4, 256) + s2c::align_up((size_t)(num_points > 0 ? num_points : 1) * 4, 256) +
           512 + s2c::align_up(s2c::scan_workspace_bytes(ns), 256) + 512;
}

extern "C" s2c_status s2c_resample_strands_by_arclength(int num_strands, const int32_t* num_samples,
                                                        const float* points, int64_t num_points, int target,
                                                        float* out, void* workspace, size_t workspace_bytes,
                                                        s2c_stream stream) {
    S2C_REQUIRE(num_strands >= 0 && num_points >= 0 && target >= 2, "resample_strands_by_arclength: bad sizes");
    S2C_REQUIRE(num_points < (1LL << 31), "resample_strands_by_arclength: too many points");
    if (num_strands == 0) return S2C_OK;
    S2C_REQUIRE(num_samples && points && out && workspace, "resample_strands_by_arclength: null pointer");
    S2C_REQUIRE(workspace_bytes >= s2c_resample_strands_workspace_size(num_strands, num_points),
                "resample_strands_by_arclength: workspace too small");
    s2c::Carver cv(workspace, workspace_bytes);
    int32_t* ends = cv.take<int32_t>(num_strands);
    int32_t* long_list = cv.take<int32_t>(num_strands);
    float* len = cv.take<float>(num_points > 0 ? num_points : 1);
    int32_t* flags = cv.take<int32_t>(2);   // [0] bad counts, [1] long strands
    void* scan = cv.take<char>(s2c::scan_workspace_bytes(num_strands));
    int64_t* tot = cv.take<int64_t>(1);
    S2C_REQUIRE(cv.ok(), "resample_strands_by_arclength: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    s2c_status s = s2c::inclusive_scan_i32(num_samples, num_strands, ends, scan, tot, st);
    if (s != S2C_OK) return s;
    cudaError_t e = cudaMemsetAsync(flags, 0, 8, st);
    if (e != cudaSuccess) return s2c::cuda_status(e, "resample_strands_by_arclength: memset");
    constexpr int threads = 32 * s2c::kResampleWarps;
    s2c::resample_warp_kernel<<<s2c::grid_for((int64_t)num_strands * 32, threads, (int64_t)s2c::num_sms() * 16),
                                threads, 0, st>>>(num_strands, num_samples, ends, points, num_points, target, out,
                                                  long_list, flags + 1, flags);
    S2C_CHECK_LAUNCH("resample_warp_kernel");
    s2c::resample_long_kernel<<<s2c::num_sms() * 2, 128, 0, st>>>(long_list, flags + 1, num_samples, ends, points,
                                                                    num_points, target, len, out);
    S2C_CHECK_LAUNCH("resample_long_kernel");
    return S2C_OK;
}
